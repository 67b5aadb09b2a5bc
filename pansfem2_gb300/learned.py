"""Host side of the learned preconditioner: the U-Net object of the C ABI
(psf_unet_*).  No counterpart in the reference, whose solvers have no learned
part; the network feeds the flexible CG of the IR_LEARNED_F32 solver."""
import ctypes as C

import numpy as np

from . import _lib as L


class UNet:
    """4-level U-Net on an H x W node grid (H, W odd), base width c0, batch
    capacity `batch`; bf16 weights/activations, fp32 accumulation, on the GPU."""

    def __init__(self, H, W, batch=1, c0=16, seed=1):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.psf_unet_create(c0, H, W, batch, seed, C.byref(h)))
        self._h, self.H, self.W, self.batch, self.c0 = h, H, W, batch, c0
        self.nparams = int(lib.psf_unet_nparams(h))

    def close(self):
        if self._h:
            L.load().psf_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _f32(a):
        return np.ascontiguousarray(a, dtype=np.float32)

    def get_params(self):
        out = np.empty(self.nparams, np.float32)
        L.check(L.load().psf_unet_get_params(self._h, L.ptr(out, C.c_float), self.nparams))
        return out

    def set_params(self, p):
        p = self._f32(p)
        L.check(L.load().psf_unet_set_params(self._h, L.ptr(p, C.c_float), p.size))

    @property
    def out_scale(self):
        v = C.c_float()
        L.check(L.load().psf_unet_get_out_scale(self._h, C.byref(v)))
        return v.value

    @out_scale.setter
    def out_scale(self, v):
        L.check(L.load().psf_unet_set_out_scale(self._h, float(v)))

    def save(self, path):
        """Parameters and output scale to an .npz file."""
        np.savez(path, params=self.get_params(), out_scale=np.float32(self.out_scale), H=self.H, W=self.W,
                 c0=self.c0)

    def load(self, path):
        d = np.load(path)
        self.set_params(d["params"])
        self.out_scale = float(d["out_scale"])

    def forward(self, inp):
        inp = self._f32(inp)
        B = inp.shape[0]
        out = np.empty((B, self.H, self.W, 2), np.float32)
        L.check(L.load().psf_unet_forward_host(self._h, B, L.ptr(inp, C.c_float), L.ptr(out, C.c_float)))
        return out

    def loss_grad(self, inp, tgt, mask=None):
        inp, tgt = self._f32(inp), self._f32(tgt)
        m = None if mask is None else self._f32(mask)
        B = inp.shape[0]
        out = np.empty((B, self.H, self.W, 2), np.float32)
        grad = np.empty(self.nparams, np.float32)
        loss = C.c_double()
        L.check(L.load().psf_unet_loss_grad_host(self._h, B, L.ptr(inp, C.c_float), L.ptr(tgt, C.c_float),
                                                 L.ptr(m, C.c_float), C.byref(loss), L.ptr(out, C.c_float),
                                                 L.ptr(grad, C.c_float)))
        return loss.value, out, grad


def conv(mode, x, w, bias=None, relu=False, out_hw=None):
    """One tensor-core convolution (psf_unet_conv): x [B,hin,win,cin], w [N,9,cin]
    -> y [B,hout,wout,N].  mode 0/1: stride 1/2; 2/3: transposed stride 1/2."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    w = np.ascontiguousarray(w, dtype=np.float32)
    B, hin, win, cin = x.shape
    N = w.shape[0]
    if out_hw is None:
        out_hw = {0: (hin, win), 1: ((hin + 1) // 2, (win + 1) // 2), 2: (hin, win),
                  3: (2 * hin - 1, 2 * win - 1)}[mode]
    hout, wout = out_hw
    y = np.empty((B, hout, wout, N), np.float32)
    b = None if bias is None else np.ascontiguousarray(bias, dtype=np.float32)
    L.check(L.load().psf_unet_conv(mode, N, cin, hin, win, hout, wout, B, L.ptr(x, C.c_float),
                                   L.ptr(w, C.c_float), L.ptr(b, C.c_float), int(relu), L.ptr(y, C.c_float)))
    return y


def bf16_round(a):
    """Round-to-nearest-even to bfloat16, returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def conv_reference(mode, x, w, bias=None, relu=False, out_hw=None):
    """float64 numpy statement of conv() on bf16-rounded inputs (test reference)."""
    x = bf16_round(x).astype(np.float64)
    w = bf16_round(w).astype(np.float64)
    B, hin, win, cin = x.shape
    N = w.shape[0]
    if out_hw is None:
        out_hw = {0: (hin, win), 1: ((hin + 1) // 2, (win + 1) // 2), 2: (hin, win),
                  3: (2 * hin - 1, 2 * win - 1)}[mode]
    hout, wout = out_hw
    y = np.zeros((B, hout, wout, N))
    oy, ox = np.meshgrid(np.arange(hout), np.arange(wout), indexing="ij")
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        if mode == 0:
            yi, xi, ok = oy + dy, ox + dx, np.ones_like(oy, bool)
        elif mode == 1:
            yi, xi, ok = 2 * oy + dy, 2 * ox + dx, np.ones_like(oy, bool)
        elif mode == 2:
            yi, xi, ok = oy - dy, ox - dx, np.ones_like(oy, bool)
        else:
            ty, tx = oy - dy, ox - dx
            ok = ((ty % 2) == 0) & ((tx % 2) == 0)
            yi, xi = ty // 2, tx // 2
        ok = ok & (yi >= 0) & (yi < hin) & (xi >= 0) & (xi < win)
        src = np.zeros((B, hout, wout, cin))
        src[:, ok] = x[:, yi[ok], xi[ok]]
        y += np.einsum("bhwc,nc->bhwn", src, w[:, t, :])
    if bias is not None:
        y += np.asarray(bias, np.float64)
    if relu:
        y = np.maximum(y, 0.0)
    return y


class TrainSet:
    """Training pairs resident on the GPU (psf_trainset_*), grid H x W nodes."""

    def __init__(self, H, W, capacity):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.psf_trainset_create(H, W, capacity, C.byref(h)))
        self._h, self.H, self.W, self.capacity = h, H, W, capacity

    def __len__(self):
        return int(L.load().psf_trainset_size(self._h))

    def close(self):
        if self._h:
            L.load().psf_trainset_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


LOSS_MODES = {"mse": 0, "energy": 1, "angle": 2}


def train(net, trainset, steps, batch=8, lr=1e-3, seed=1, loss="energy"):
    """Adam on the GPU (psf_learned_train); returns the loss per step relative to
    that of a zero output (loss: "angle" = K-norm error left by the best multiple of
    the correction, "energy" = K-norm error, "mse" = squared error)."""
    hist = np.zeros(steps)
    L.check(L.load().psf_learned_train(net._h, trainset._h, int(steps), int(batch), float(lr), int(seed),
                                       LOSS_MODES[loss], L.ptr(hist)))
    return hist


def evaluate(net, trainset, first=0, count=None, optimal_step=True):
    """Mean energy-norm error of the network's correction over pairs
    [first, first + count), relative to no correction (1 = no gain); with the
    energy-optimal step the solver applies (default) or as output."""
    count = len(trainset) - first if count is None else count
    v = C.c_double()
    L.check(L.load().psf_learned_eval(net._h, trainset._h, int(first), int(count), 2 if optimal_step else 1,
                                      C.byref(v)))
    return v.value
