"""GPU checks of the learned preconditioner's network kernels.

* One tensor-core convolution (tcgen05 implicit GEMM) in every gather mode and
  every channel count the network uses, against a float64 numpy statement:
  bit-exact on integer data (every partial sum exact in fp32), ~1e-6 relative on
  random data (fp32 accumulation order).
* The whole network, forward and backward, against the CPU oracle
  (oracle/unet_oracle.c with bf16 rounding at the same points): output,
  loss and the gradient of every layer's weights and biases.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from pansfem2_gb300 import learned as Ln

pytestmark = pytest.mark.gpu

NC = [(16, 8), (32, 16), (48, 32), (64, 64), (96, 32), (128, 128), (192, 64), (16, 192)]


def _grid(mode):
    # output grid 9 x 13 for every mode (the transposed stride-2 mode reads a 5 x 7 grid)
    return {0: (9, 13), 1: (17, 25), 2: (9, 13), 3: (5, 7)}[mode]


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
@pytest.mark.parametrize("N,cin", NC)
def test_conv_exact_on_integers(mode, N, cin):
    rng = np.random.default_rng(10 * mode + N + cin)
    h, w = _grid(mode)
    x = rng.integers(-4, 5, (2, h, w, cin)).astype(np.float32)
    wt = rng.integers(-4, 5, (N, 9, cin)).astype(np.float32)
    bias = rng.integers(-8, 9, N).astype(np.float32)
    out_hw = (9, 13)
    y = Ln.conv(mode, x, wt, bias, relu=False, out_hw=out_hw)
    ref = Ln.conv_reference(mode, x, wt, bias, relu=False, out_hw=out_hw)
    assert np.array_equal(y.astype(np.float64), ref), np.argwhere(y != ref)[:5]


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
@pytest.mark.parametrize("N,cin", [(16, 8), (64, 64), (128, 128), (192, 64)])
def test_conv_random_many_tiles(mode, N, cin):
    rng = np.random.default_rng(7 + mode)
    hout, wout = 65, 97
    hin, win = {0: (65, 97), 1: (129, 193), 2: (65, 97), 3: (33, 49)}[mode]
    x = rng.standard_normal((2, hin, win, cin)).astype(np.float32)
    wt = (rng.standard_normal((N, 9, cin)) / np.sqrt(9 * cin)).astype(np.float32)
    bias = rng.standard_normal(N).astype(np.float32)
    y = Ln.conv(mode, x, wt, bias, relu=True, out_hw=(hout, wout))
    ref = Ln.conv_reference(mode, x, wt, bias, relu=True, out_hw=(hout, wout))
    err = np.abs(y - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def _net_case(seed, B, H, W):
    rng = np.random.default_rng(seed)
    inp = np.zeros((B, H, W, 8), np.float32)
    inp[..., 0] = rng.random((B, H, W))
    inp[..., 1:3] = rng.standard_normal((B, H, W, 2))
    tgt = rng.standard_normal((B, H, W, 2)).astype(np.float32)
    mask = (rng.random((B, H, W, 2)) > 0.05).astype(np.float32)
    return inp, tgt, mask


def _layer_slices(c0=16):
    layers = [(8, c0), (c0, c0), (c0, 2 * c0), (2 * c0, 2 * c0), (2 * c0, 4 * c0), (4 * c0, 4 * c0),
              (4 * c0, 8 * c0), (8 * c0, 8 * c0), (12 * c0, 4 * c0), (4 * c0, 4 * c0), (6 * c0, 2 * c0),
              (2 * c0, 2 * c0), (3 * c0, c0), (c0, c0), (c0, 2)]
    out, off = [], 0
    for cin, cout in layers:
        out.append((slice(off, off + 9 * cin * cout), slice(off + 9 * cin * cout, off + 9 * cin * cout + cout)))
        off += 9 * cin * cout + cout
    return out


@pytest.mark.parametrize("B,H,W", [(2, 17, 33), (1, 65, 33)])
def test_network_forward_backward_vs_oracle(B, H, W):
    inp, tgt, mask = _net_case(B * H + W, B, H, W)
    with Ln.UNet(H, W, batch=B, seed=5) as net:
        params = net.get_params()
        assert params.size == O.unet_nparams(16)
        loss, out, grad = net.loss_grad(inp, tgt, mask)
        out_f = net.forward(inp)
    l_ref, o_ref, g_ref = O.unet_loss_grad(params, inp, tgt, mask, bf16=True)
    assert np.array_equal(out, out_f)
    e_out = np.linalg.norm(out - o_ref) / np.linalg.norm(o_ref)
    assert e_out < 1e-2, e_out
    assert abs(loss - l_ref) <= 1e-3 * abs(l_ref), (loss, l_ref)
    for k, (ws, bs) in enumerate(_layer_slices()):
        for s, what in ((ws, "W"), (bs, "b")):
            e = np.linalg.norm(grad[s] - g_ref[s]) / max(np.linalg.norm(g_ref[s]), 1e-30)
            # a bf16 rounding flip (0.4 %) of one stored activation or gradient propagates through every
            # later product; the flips accumulate along the backward chain, whose end is the first layer.
            # A wrong index or layout gives errors of order 1.
            assert e < (8e-2 if k == 0 else 5e-2), (k, what, e)


def test_network_params_roundtrip_and_batch_limit():
    with Ln.UNet(9, 9, batch=2, seed=3) as net:
        p = net.get_params()
        p2 = p * 0.5
        net.set_params(p2)
        assert np.array_equal(net.get_params(), p2)
        inp, _, _ = _net_case(1, 3, 9, 9)
        with pytest.raises(Exception):
            net.forward(inp)   # batch 3 > capacity 2
