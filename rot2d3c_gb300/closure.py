"""Learned subgrid closure over the C-ABI (r2d3c_cnn_*): the CNN and its
training, on device tensors (torch CUDA tensors or raw device pointers)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, load

CIN = [8, 32, 32, 32, 32, 32]
COUT = [32, 32, 32, 32, 32, 2]


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t if isinstance(t, int) else t.data_ptr())


def _ready(*ts) -> None:
    """The library's kernels run on their own non-blocking streams, which do
    not wait for torch's: before a call reads or writes torch tensors, the
    work torch has queued on them must be complete."""
    for t in ts:
        if t is not None and not isinstance(t, int):
            import torch
            torch.cuda.current_stream(t.device).synchronize()
            return


class CNN:
    """The closure network on an H x W periodic grid (see include/r2d3c.h)."""

    def __init__(self, H: int, W: int, max_batch: int, seed: int = 0):
        self.H, self.W, self.max_batch = H, W, max_batch
        h = C.c_void_p()
        check(load().r2d3c_cnn_create(H, W, max_batch, seed, C.byref(h)), "cnn_create")
        self._h = h
        n = C.c_longlong()
        check(load().r2d3c_cnn_num_params(self._h, C.byref(n)), "cnn_num_params")
        self.nparams = n.value

    def get_params(self) -> np.ndarray:
        out = np.empty(self.nparams, np.float32)
        check(load().r2d3c_cnn_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float))), "cnn_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        check(load().r2d3c_cnn_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))), "cnn_set_params")

    def set_normalization(self, in_mean, in_std, out_mean, out_std) -> None:
        arrs = [np.ascontiguousarray(a, np.float32) for a in (in_mean, in_std, out_mean, out_std)]
        ptrs = [a.ctypes.data_as(C.POINTER(C.c_float)) for a in arrs]
        check(load().r2d3c_cnn_set_normalization(self._h, *ptrs), "cnn_set_normalization")

    def forward(self, x, batch: int, out) -> None:
        _ready(x, out)
        check(load().r2d3c_cnn_forward(self._h, _ptr(x), batch, _ptr(out)), "cnn_forward")

    def gradients(self, x, y, batch: int):
        g = np.empty(self.nparams, np.float32)
        loss = C.c_double()
        _ready(x, y)
        check(load().r2d3c_cnn_gradients(self._h, _ptr(x), _ptr(y), batch, g.ctypes.data_as(C.POINTER(C.c_float)),
                                         C.byref(loss)), "cnn_gradients")
        return loss.value, g

    def backward(self, x, gout, batch: int, gx=None):
        """Vector-Jacobian product at x (r2d3c_cnn_backward): dL/dx into gx
        (optional) for dL/d(output) = gout; returns dL/dparams."""
        g = np.empty(self.nparams, np.float32)
        _ready(x, gout, gx)
        check(load().r2d3c_cnn_backward(self._h, _ptr(x), _ptr(gout), batch, None if gx is None else _ptr(gx),
                                        g.ctypes.data_as(C.POINTER(C.c_float))), "cnn_backward")
        return g

    def train_step(self, x, y, batch: int, lr: float = 1e-3) -> float:
        loss = C.c_double()
        _ready(x, y)
        check(load().r2d3c_cnn_train_step(self._h, _ptr(x), _ptr(y), batch, lr, C.byref(loss)), "cnn_train_step")
        return loss.value

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            load().r2d3c_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def closure_inputs(ctx, d_x) -> None:
    """The 8 network inputs of ctx's current state into d_x ([n, n, 8] FP32)."""
    _ready(d_x)
    check(load().r2d3c_closure_inputs(ctx._h, _ptr(d_x)), "closure_inputs")


def closure_sample(fine, coarse, d_x, d_y) -> None:
    """Filter fine's state onto coarse; inputs and subgrid targets of it."""
    _ready(d_x, d_y)
    check(load().r2d3c_closure_sample(fine._h, coarse._h, _ptr(d_x), _ptr(d_y)), "closure_sample")


def set_tendency(ctx, d_t) -> None:
    """Subgrid tendencies ([n, n, 2] FP32, physical) added to the brackets of
    the following steps of ctx; None switches them off."""
    _ready(d_t)
    check(load().r2d3c_closure_set_tendency(ctx._h, None if d_t is None else _ptr(d_t)), "closure_set_tendency")


def set_band(ctx, w) -> None:
    """Per-shell weights of ctx's learned tendencies (r2d3c_closure_set_band):
    ``w`` is [2, nshells] (omega tendency, vz tendency) or None (off)."""
    if w is None:
        check(load().r2d3c_closure_set_band(ctx._h, None, 0), "closure_set_band")
        return
    w = np.ascontiguousarray(w, np.float32)
    assert w.ndim == 2 and w.shape[0] == 2
    check(load().r2d3c_closure_set_band(ctx._h, C.c_void_p(w.ctypes.data), w.shape[1]), "closure_set_band")


def shell_index(n: int) -> np.ndarray:
    """Shell kmn = int(sqrt(ka2) + .5) of every element of an [kx][ky]
    spectral plane of an n^2 grid (the engine's shell rule)."""
    h = n // 2
    ka = np.concatenate([np.arange(h), np.arange(h) - h]).astype(np.float64)
    k2 = ka[: h + 1, None] ** 2 + ka[None, :] ** 2
    return np.floor(np.sqrt(k2) + 0.5).astype(np.int64)


def band_fit(net: CNN, X, Y, idx, n: int, batch: int = 8):
    """Per-shell skill of the network on the snapshots ``idx`` (held-out
    data): for each tendency c and shell b the least-squares weight
    w = sum Re(P conj T) / sum |P|^2 over the shell's modes, clipped to
    [0, 1], where P and T are the spectra of the prediction and of the
    target; shells where the prediction is uncorrelated with the target get
    weights near 0.  The spectra come from the library's own FP64 transform
    on the device.  Returns [2, n/2+1] float32."""
    import torch
    from . import FP64, R2C, FFTPlan
    batch = max(1, min(batch, net.max_batch))
    nb = n // 2 + 1
    sh = shell_index(n)
    two = np.full(sh.shape, 2.0)
    two[0] = 1.0
    keep = sh < nb  # the corners beyond shell n/2 lie outside every retained mode
    sh, two = sh[keep], two[keep]
    num = np.zeros((2, nb))
    den = np.zeros((2, nb))
    plan = FFTPlan(n, R2C, FP64)
    out = torch.empty((batch, n, n, 2), dtype=torch.float32, device="cuda")
    phys = torch.empty((n, n), dtype=torch.float64, device="cuda")
    spec = torch.empty((nb, n, 2), dtype=torch.float64, device="cuda")

    def r2c(field):
        phys.copy_(field)
        plan.r2c_dev(phys.data_ptr(), spec.data_ptr(), torch.cuda.current_stream().cuda_stream)
        s = spec.cpu().numpy()
        return (s[..., 0] + 1j * s[..., 1])[keep]
    idx = list(idx)
    for i0 in range(0, len(idx), batch):
        ids = idx[i0:i0 + batch]
        xb = X[ids].contiguous()
        net.forward(xb, len(ids), out)
        torch.cuda.synchronize()
        for j, i in enumerate(ids):
            for c in range(2):
                P = r2c(out[j, :, :, c])
                T = r2c(Y[i, :, :, c])
                num[c] += np.bincount(sh, two * (P * np.conj(T)).real, minlength=nb)
                den[c] += np.bincount(sh, two * np.abs(P) ** 2, minlength=nb)
    plan.destroy()
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(den > 0, num / den, 0.0)
    return np.clip(w, 0.0, 1.0).astype(np.float32)


def closure_advance(ctx, net: CNN, nsteps: int, dt_mode: int, cfl_or_dt: float, every: int = 1,
                    overlap: bool = False):
    """nsteps LES steps of ctx with the network evaluated before every step
    (``every`` > 1: before every every-th step, its tendencies held in
    between; one captured CUDA graph per evaluation and its steps).  With
    ``overlap`` the network runs one step behind, beside the step (step s > 0
    takes the tendencies of the state before step s - 1;
    r2d3c_closure_advance_overlapped).  Returns (time, dt of the last step)."""
    t, dtl = C.c_double(), C.c_double()
    if overlap:
        if every != 1:
            raise ValueError("overlap takes every = 1")
        check(load().r2d3c_closure_advance_overlapped(ctx._h, net._h, nsteps, dt_mode, cfl_or_dt, C.byref(t),
                                                      C.byref(dtl)), "closure_advance_overlapped")
    elif every == 1:
        check(load().r2d3c_closure_advance(ctx._h, net._h, nsteps, dt_mode, cfl_or_dt, C.byref(t), C.byref(dtl)),
              "closure_advance")
    else:
        check(load().r2d3c_closure_advance_every(ctx._h, net._h, nsteps, every, dt_mode, cfl_or_dt, C.byref(t),
                                                 C.byref(dtl)), "closure_advance_every")
    return t.value, dtl.value
