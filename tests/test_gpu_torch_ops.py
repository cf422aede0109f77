"""The PyTorch binding of the closure network (rot2d3c::cnn_forward, a
torch.library custom operator over r2d3c_cnn_forward / r2d3c_cnn_backward):
its autograd gradients against the float64 oracle's vector-Jacobian product,
and a PyTorch optimiser step that changes the network the C-ABI runs."""
import numpy as np
import pytest

from oracle import cnn_oracle as CO
from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu


def test_autograd_matches_the_oracle_vjp(gpu):
    import torch
    from rot2d3c_gb300.torch_ops import ClosureNet
    H, W, B = 8, 16, 2
    m = ClosureNet(H, W, B, seed=5)
    rng = np.random.default_rng(4)
    im, isd = rng.standard_normal(8).astype(np.float32), rng.uniform(0.5, 2, 8).astype(np.float32)
    om, osd = rng.standard_normal(2).astype(np.float32), rng.uniform(0.5, 2, 2).astype(np.float32)
    m.set_normalization(im, isd, om, osd)
    x = (rng.standard_normal((B, H, W, 8)) * 2).astype(np.float32)
    wl = rng.standard_normal((B, H, W, 2)).astype(np.float32)  # loss = sum(out * wl)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    out = m(xt)
    loss = (out * torch.from_numpy(wl).cuda()).sum()
    loss.backward()
    p = m.params.detach().cpu().numpy().astype(np.float64)
    xs = (x - im) / isd
    pre, _, _ = CO.forward(p, xs)
    np.testing.assert_allclose(out.detach().cpu().numpy(), pre * osd + om, rtol=0,
                               atol=1e-2 * np.abs(pre * osd + om).max())
    gp, gxs = CO.vjp(p, xs, wl * osd)
    gx = gxs[..., :8] / isd
    assert rel_l2(m.params.grad.cpu().numpy(), gp) < 3e-2
    assert rel_l2(xt.grad.cpu().numpy(), gx) < 3e-2


def test_optimiser_step_reaches_the_network(gpu):
    import torch
    from rot2d3c_gb300.torch_ops import ClosureNet
    H, W, B = 8, 16, 1
    m = ClosureNet(H, W, B, seed=6)
    x = torch.randn((B, H, W, 8), device="cuda")
    y0 = m(x).detach().clone()
    loss = (m(x) ** 2).mean()
    loss.backward()
    # a step that the linearisation says lowers the loss by 5%
    g2 = float((m.params.grad ** 2).sum())
    opt = torch.optim.SGD(m.parameters(), lr=0.05 * float(loss) / g2)
    opt.step()
    y1 = m(x).detach()
    assert float((y1 ** 2).mean()) < float((y0 ** 2).mean())
    # the C-ABI network itself now holds the optimiser's parameters
    np.testing.assert_array_equal(m.net.get_params(), m.params.detach().cpu().numpy())
