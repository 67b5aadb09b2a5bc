"""CPU checks of the U-Net oracle (the checker of the GPU network kernels):
its backward pass against central finite differences in double precision, the
bf16 emulation staying close to the exact network, and the parameter count of
the 4-level, 16->128-channel configuration."""
import numpy as np
import pytest

from oracle import pyoracle as O


LAYERS = [(8, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128),
          (192, 64), (64, 64), (96, 32), (32, 32), (48, 16), (16, 16), (16, 2)]


def he_params(rng, layers=LAYERS):
    """He-normal weights (std sqrt(2 / (9 cin))), small random biases."""
    out = []
    for cin, cout in layers:
        out.append(rng.standard_normal(9 * cin * cout) * np.sqrt(2.0 / (9 * cin)))
        out.append(rng.standard_normal(cout) * 0.05)
    return np.concatenate(out).astype(np.float32)


def _case(seed, B=2, H=9, W=17, c0=16):
    rng = np.random.default_rng(seed)
    params = he_params(rng)
    inp = np.zeros((B, H, W, 8), np.float32)
    inp[..., :3] = rng.standard_normal((B, H, W, 3))
    tgt = rng.standard_normal((B, H, W, 2)).astype(np.float32)
    mask = (rng.random((B, H, W, 2)) > 0.1).astype(np.float32)
    return params, inp, tgt, mask


def test_parameter_count():
    # per layer 9*cin*cout + cout, channels 16, 32, 64, 128, inputs padded to 8
    assert O.unet_nparams(16) == sum(9 * a * b + b for a, b in LAYERS)


def test_gradient_matches_finite_differences():
    params, inp, tgt, mask = _case(0)
    loss, _, grad = O.unet_loss_grad(params, inp, tgt, mask, bf16=False)
    assert np.isfinite(loss) and np.abs(grad).max() > 0
    rng = np.random.default_rng(1)
    # check the largest gradients and a random sample, in every layer
    idx = np.unique(np.concatenate([np.argsort(-np.abs(grad))[:40], rng.choice(params.size, 60, replace=False)]))
    h = 1e-4
    bad = []
    for i in idx:
        p1 = params.copy()
        p2 = params.copy()
        p1[i] += np.float32(h)
        p2[i] -= np.float32(h)
        d1 = float(p1[i]) - float(params[i])
        d2 = float(params[i]) - float(p2[i])
        l1, _, _ = O.unet_loss_grad(p1, inp, tgt, mask, bf16=False, want_grad=False)
        l2, _, _ = O.unet_loss_grad(p2, inp, tgt, mask, bf16=False, want_grad=False)
        fd = (l1 - l2) / (d1 + d2)
        if abs(fd - grad[i]) > 2e-3 * max(abs(grad[i]), 1e-2 * np.abs(grad).max()):
            bad.append((int(i), fd, float(grad[i])))
    # a ReLU kink inside +-h can spoil an isolated entry; nothing systematic
    assert len(bad) <= 2, bad


def test_bf16_emulation_close_to_exact():
    params, inp, tgt, mask = _case(2)
    l0, o0, g0 = O.unet_loss_grad(params, inp, tgt, mask, bf16=False)
    l1, o1, g1 = O.unet_loss_grad(params, inp, tgt, mask, bf16=True)
    assert abs(l1 - l0) <= 2e-2 * abs(l0)
    assert np.linalg.norm(o1 - o0) <= 3e-2 * np.linalg.norm(o0)
    assert np.linalg.norm(g1 - g0) <= 5e-2 * np.linalg.norm(g0)


@pytest.mark.parametrize("shape", [(1, 9, 9), (3, 17, 9)])
def test_shapes_and_mask(shape):
    B, H, W = shape
    params, inp, tgt, mask = _case(3, B, H, W)
    loss, out, grad = O.unet_loss_grad(params, inp, tgt, np.zeros_like(mask), bf16=True)
    # an all-zero mask gives zero loss and zero gradient
    assert loss == 0.0 and not grad.any() and out.shape == (B, H, W, 2)
