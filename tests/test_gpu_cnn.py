"""The closure CNN's tensor-core kernels against the float64 NumPy reference:
forward outputs, loss and every parameter gradient (the reference emulates
the bfloat16 rounding of operands, so the comparison isolates accumulation
order), and a training run that lowers the loss."""
import numpy as np
import pytest

from oracle import cnn_oracle as CO

pytestmark = pytest.mark.gpu


def _layer_slices():
    out, off = [], 0
    for ci, co in zip(CO.CIN, CO.COUT):
        out.append((slice(off, off + 9 * ci * co), slice(off + 9 * ci * co, off + 9 * ci * co + co)))
        off += 9 * ci * co + co
    return out


@pytest.mark.parametrize("H,W,B", [(8, 16, 2), (16, 32, 1), (8, 128, 2), (8, 256, 1)])
def test_forward_and_gradients_match_reference(gpu, H, W, B):
    import torch
    from rot2d3c_gb300.closure import CNN
    net = CNN(H, W, B, seed=3)
    rng = np.random.default_rng(H + W)
    params = net.get_params()
    # non-zero biases so their gradients and broadcasts are exercised
    for _, bs in _layer_slices():
        params[bs] = rng.uniform(-0.1, 0.1, bs.stop - bs.start)
    net.set_params(params)
    x = rng.standard_normal((B, H, W, 8)).astype(np.float32)
    t = rng.standard_normal((B, H, W, 2)).astype(np.float32) * 0.1
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    out = torch.empty((B, H, W, 2), dtype=torch.float32, device="cuda")
    net.forward(dx, B, out)
    ref_out, _, _ = CO.forward(params.astype(np.float64), x.astype(np.float64))
    o = out.cpu().numpy()
    assert np.linalg.norm(o - ref_out) <= 1e-2 * np.linalg.norm(ref_out)
    loss, g = net.gradients(dx, dt, B)
    ref_loss, ref_g = CO.loss_and_grads(params.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss
    for l, (ws, bs) in enumerate(_layer_slices()):
        for sl in (ws, bs):
            a, b = g[sl], ref_g[sl]
            assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-12, (l, np.linalg.norm(a - b) / np.linalg.norm(b))


def test_training_lowers_the_loss(gpu):
    """Learn a fixed periodic stencil of the inputs (a target the network can
    represent): the loss falls by an order of magnitude."""
    import torch
    from rot2d3c_gb300.closure import CNN
    H, W, B = 32, 32, 4
    net = CNN(H, W, B, seed=1)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((B, H, W, 8)).astype(np.float32)
    lap = np.roll(x, 1, 1) + np.roll(x, -1, 1) + np.roll(x, 1, 2) + np.roll(x, -1, 2) - 4 * x
    t = np.stack([lap[..., 0] + 0.5 * x[..., 3], x[..., 1] * 0.7 - lap[..., 5]], axis=-1).astype(np.float32)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = net.train_step(dx, dt, B, 3e-3)
    for _ in range(300):
        last = net.train_step(dx, dt, B, 3e-3)
    assert np.isfinite(last) and last < 0.1 * first


def test_tensor_core_convolutions_match_the_warp_mma_ones(gpu, monkeypatch):
    """W % 128 == 0 runs the tcgen05 convolutions (TMEM accumulators); the
    same network with R2D3C_CNN_CONV=mma runs the warp-level MMA kernels:
    outputs, loss and gradients agree to the accumulation-order level."""
    import torch
    from rot2d3c_gb300.closure import CNN
    H, W, B = 16, 256, 2
    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.standard_normal((B, H, W, 8)).astype(np.float32)).cuda()
    t = torch.from_numpy((0.1 * rng.standard_normal((B, H, W, 2))).astype(np.float32)).cuda()
    res = []
    for mode in ("tcgen05", "mma"):
        monkeypatch.setenv("R2D3C_CNN_CONV", mode)
        net = CNN(H, W, B, seed=9)
        out = torch.empty((B, H, W, 2), dtype=torch.float32, device="cuda")
        net.forward(x, B, out)
        loss, g = net.gradients(x, t, B)
        res.append((out.cpu().numpy(), loss, g))
    (o1, l1, g1), (o2, l2, g2) = res
    assert np.linalg.norm(o1 - o2) <= 1e-2 * np.linalg.norm(o2)
    assert abs(l1 - l2) <= 1e-3 * l2
    assert np.linalg.norm(g1 - g2) <= 1e-2 * np.linalg.norm(g2)
