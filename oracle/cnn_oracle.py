"""Float64 NumPy reference of the closure CNN (TEST INFRASTRUCTURE ONLY).

Six periodic 3x3 convolutions 8 -> 32 -> 32 -> 32 -> 32 -> 32 -> 2 with
GELU (erf form) between them, NHWC layout, MSE loss, and the hand-derived
backward pass.  With ``emulate=True`` the inputs, weights, inter-layer
activations and back-propagated gradients are rounded to bfloat16 where the
GPU kernels round them, so the comparison isolates accumulation order.
The network has no counterpart in the reference program.
"""
import numpy as np
from scipy.special import erf

CIN = [8, 32, 32, 32, 32, 32]
COUT = [32, 32, 32, 32, 32, 2]


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    a = (a + 0x7FFF + ((a >> 16) & 1)) & 0xFFFF0000
    return a.astype(np.uint32).view(np.float32).astype(np.float64)


def split(params):
    """Flat parameter vector -> [(w [9,cin,cout], b [cout])] per layer."""
    out, off = [], 0
    for ci, co in zip(CIN, COUT):
        w = params[off:off + 9 * ci * co].reshape(9, ci, co).astype(np.float64)
        off += 9 * ci * co
        b = params[off:off + co].astype(np.float64)
        off += co
        out.append((w, b))
    return out


def conv(x, w):
    """y[b,i,j] = sum_tap x[b, i+dy-1, j+dx-1] @ w[tap], periodic."""
    y = np.zeros(x.shape[:3] + (w.shape[2],))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        y += np.roll(x, shift=(-(dy - 1), -(dx - 1)), axis=(1, 2)) @ w[tap]
    return y


def conv_t(g, w):
    """Adjoint of conv: dx[b,q] = sum_tap g[b, q - off(tap)] @ w[tap]^T."""
    x = np.zeros(g.shape[:3] + (w.shape[1],))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        x += np.roll(g, shift=(dy - 1, dx - 1), axis=(1, 2)) @ w[tap].T
    return x


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(params, x, emulate=True):
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    layers = split(params)
    a = r(x)
    acts, pres = [a], []
    for l, (w, b) in enumerate(layers):
        y = conv(a, r(w)) + b
        pres.append(y)
        if l < len(layers) - 1:
            a = r(gelu(y))
            acts.append(a)
    return pres[-1], acts, pres


def loss_and_grads(params, x, t, emulate=True):
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    layers = split(params)
    out, acts, pres = forward(params, x, emulate)
    cnt = out.size
    loss = float(np.sum((out - t) ** 2) / cnt)
    g = r(2.0 * (out - t) / cnt)
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        w, b = layers[l]
        a = acts[l]
        dw = np.zeros_like(w)
        for tap in range(9):
            dy, dx = divmod(tap, 3)
            xs = np.roll(a, shift=(-(dy - 1), -(dx - 1)), axis=(1, 2))
            dw[tap] = np.einsum("bijc,bijo->co", xs, g)
        db = g.sum(axis=(0, 1, 2))
        grads[l] = (dw, db)
        if l == 0:
            break
        da = r(conv_t(g, r(w)))
        g = r(da * gelu_d(pres[l - 1]))
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return loss, flat


def vjp(params, x, g_out, emulate=True):
    """Vector-Jacobian product of the network at the (standardised) input x
    for dL/d(output) = g_out: returns (dL/dparams flat, dL/dx), rounding to
    bfloat16 where the GPU kernels round (the output gradient, every
    back-propagated activation gradient)."""
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    layers = split(params)
    out, acts, pres = forward(params, x, emulate)
    g = r(g_out)
    grads = [None] * len(layers)
    dx = None
    for l in range(len(layers) - 1, -1, -1):
        w, b = layers[l]
        a = acts[l]
        dw = np.zeros_like(w)
        for tap in range(9):
            dy, dx_ = divmod(tap, 3)
            xs = np.roll(a, shift=(-(dy - 1), -(dx_ - 1)), axis=(1, 2))
            dw[tap] = np.einsum("bijc,bijo->co", xs, g)
        grads[l] = (dw, g.sum(axis=(0, 1, 2)))
        da = r(conv_t(g, r(w)))
        if l == 0:
            dx = da
            break
        g = r(da * gelu_d(pres[l - 1]))
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return flat, dx
