"""The learned-closure data path against the oracle: sharp spectral filter of
a fine run onto a coarse grid, the 8 network inputs, the subgrid bracket
targets, and the RK step with tendencies added to the brackets."""
import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import params, random_forcing, random_state, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-5)])
def test_closure_sample_matches_oracle(gpu, prec, tol):
    import torch
    from rot2d3c_gb300.closure import closure_sample
    nf, nc = 64, 32
    gf, gc = O.Grid(nf), O.Grid(nc)
    _, cpf = params(nf, iflow=0)
    _, cpc = params(nc, iflow=0)
    _, psf, vzf = random_state(nf, 5, amp=4.0)
    fine, coarse = gpu.Context(cpf, prec), gpu.Context(cpc, prec)
    fine.set_state(psf, vzf)
    dx = torch.zeros((nc, nc, 8), dtype=torch.float32, device="cuda")
    dy = torch.zeros((nc, nc, 2), dtype=torch.float32, device="cuda")
    closure_sample(fine, coarse, dx, dy)
    a, b = coarse.get_state()
    assert rel_l2(a, O.coarsen(gf, gc, psf)) < tol and rel_l2(b, O.coarsen(gf, gc, vzf)) < tol
    x = O.closure_inputs(gc, O.coarsen(gf, gc, psf), O.coarsen(gf, gc, vzf))
    t = O.closure_targets(gf, gc, psf, vzf)
    xs, ts = dx.cpu().numpy(), dy.cpu().numpy()
    ftol = max(tol, 2e-6)  # channels are stored in FP32
    for c in range(8):
        assert rel_l2(xs[..., c], x[..., c]) < ftol, c
    for c in range(2):
        assert rel_l2(ts[..., c], t[..., c]) < 10 * ftol, c


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_step_with_subgrid_tendencies(gpu, prec, tol):
    import torch
    from rot2d3c_gb300.closure import set_tendency
    n = 32
    p, cp = params(n, omega=1.0, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 8, amp=10.0)
    fp, fz = random_forcing(g, 9)
    rng = np.random.default_rng(2)
    t = np.stack([O.c2r(g, O.random_phase_field(g, 1, 10, -1.0, rng)) for _ in range(2)], axis=-1)
    t = (t / n**2 * 1e3).astype(np.float32)
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    set_tendency(c, torch.from_numpy(t).cuda())
    c.step(1e-3)
    c.advance(2, gpu.DT_FIXED, 1e-3)
    tau5 = O.r2c(g, t[..., 0].astype(np.float64))
    tau6 = O.r2c(g, t[..., 1].astype(np.float64))
    for _ in range(3):
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, 1e-3, tau5=tau5, tau6=tau6)
    a, b = c.get_state()
    assert rel_l2(a, ps) < tol and rel_l2(b, vz) < tol
    set_tendency(c, None)


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_band_weights_scale_each_shell_of_the_tendencies(gpu, prec, tol):
    """r2d3c_closure_set_band: the tendencies enter the step multiplied per
    shell by the omega / vz weights (0 beyond the weighted shells)."""
    import torch
    from rot2d3c_gb300.closure import set_band, set_tendency, shell_index
    n = 32
    p, cp = params(n, omega=1.0, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 18, amp=10.0)
    fp, fz = random_forcing(g, 19)
    rng = np.random.default_rng(3)
    t = np.stack([O.c2r(g, O.random_phase_field(g, 1, 12, -1.0, rng)) for _ in range(2)], axis=-1)
    t = (t / n**2 * 1e3).astype(np.float32)
    nw = 10  # shells 10 and beyond get weight 0
    w = rng.uniform(0.0, 1.0, (2, nw)).astype(np.float32)
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    set_band(c, w)
    set_tendency(c, torch.from_numpy(t).cuda())
    c.advance(2, gpu.DT_FIXED, 1e-3)
    sh = shell_index(n)
    fac = [np.where(sh < nw, w[k][np.minimum(sh, nw - 1)].astype(np.float64), 0.0) for k in range(2)]
    tau5 = fac[0] * O.r2c(g, t[..., 0].astype(np.float64))
    tau6 = fac[1] * O.r2c(g, t[..., 1].astype(np.float64))
    for _ in range(2):
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, 1e-3, tau5=tau5, tau6=tau6)
    a, b = c.get_state()
    assert rel_l2(a, ps) < tol and rel_l2(b, vz) < tol, (rel_l2(a, ps), rel_l2(b, vz))
    set_tendency(c, None)
    set_band(c, None)


def test_cnn_normalisation_maps_units(gpu):
    import torch
    from oracle import cnn_oracle as CO
    from rot2d3c_gb300.closure import CNN
    H, W = 8, 16
    net = CNN(H, W, 1, seed=4)
    rng = np.random.default_rng(1)
    im, isd = rng.standard_normal(8).astype(np.float32), rng.uniform(0.5, 2, 8).astype(np.float32)
    om, osd = rng.standard_normal(2).astype(np.float32), rng.uniform(0.5, 2, 2).astype(np.float32)
    net.set_normalization(im, isd, om, osd)
    x = rng.standard_normal((1, H, W, 8)).astype(np.float32) * 3
    out = torch.empty((1, H, W, 2), dtype=torch.float32, device="cuda")
    net.forward(torch.from_numpy(x).cuda(), 1, out)
    ref, _, _ = CO.forward(net.get_params().astype(np.float64), (x - im) / isd)
    ref = ref * osd + om
    assert np.linalg.norm(out.cpu().numpy() - ref) <= 1e-2 * np.linalg.norm(ref)


@pytest.mark.parametrize("prec,band", [(0, False), (1, False), (1, True)])
def test_graph_captured_les_steps_equal_the_step_by_step_loop(gpu, prec, band):
    """r2d3c_closure_advance (inputs, network, tendencies and the RK step in
    one captured graph) gives bit-identical states to the same steps made one
    call at a time, in both dt modes, with and without per-shell weights;
    the tendencies are off afterwards."""
    import torch
    from rot2d3c_gb300.closure import CNN, closure_advance, closure_inputs, set_band, set_tendency
    n = 32
    _, cp = params(n, omega=1.0, nu=2e-3, nuv=2e-3, hnu=0.1, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 41, amp=20.0)
    fp, fz = random_forcing(g, 42, 2.0, 4.0)
    net = CNN(n, n, 1, 7)
    net.set_normalization(np.zeros(8), np.full(8, 50.0), np.zeros(2), np.full(2, 5.0))
    for mode, val in ((gpu.DT_CFL, 0.4), (gpu.DT_FIXED, 1e-3)):
        a = gpu.Context(cp, prec)
        b = gpu.Context(cp, prec)
        for c in (a, b):
            c.set_state(ps, vz)
            c.set_forcing(fp, fz)
            c.set_time(0.0)
            if band:
                set_band(c, np.linspace(1.0, 0.2, 2 * 12, dtype=np.float32).reshape(2, 12))
        x = torch.empty((1, n, n, 8), dtype=torch.float32, device="cuda")
        t = torch.empty((1, n, n, 2), dtype=torch.float32, device="cuda")
        for _ in range(5):
            closure_inputs(a, x[0])
            net.forward(x, 1, t)
            set_tendency(a, t[0])
            ta, _ = a.advance(1, mode, val)
        set_tendency(a, None)
        tb, _ = closure_advance(b, net, 3, mode, val)
        tb, _ = closure_advance(b, net, 2, mode, val)
        assert ta == tb
        for u, v in zip(a.get_state(), b.get_state()):
            np.testing.assert_array_equal(u, v)
        # tendencies off: plain steps agree again
        a.advance(2, mode, val)
        b.advance(2, mode, val)
        for u, v in zip(a.get_state(), b.get_state()):
            np.testing.assert_array_equal(u, v)


@pytest.mark.parametrize("prec", [0, 1])
def test_network_every_second_step_equals_the_step_by_step_loop(gpu, prec):
    """r2d3c_closure_advance_every with every = 2: the network evaluated
    before every second step and its tendencies held for two steps, in one
    graph per pair of steps; bit-identical to the same schedule made one
    call at a time."""
    import torch
    from rot2d3c_gb300.closure import CNN, closure_advance, closure_inputs, set_tendency
    n = 32
    _, cp = params(n, omega=1.0, nu=2e-3, nuv=2e-3, hnu=0.1, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 51, amp=20.0)
    fp, fz = random_forcing(g, 52, 2.0, 4.0)
    net = CNN(n, n, 1, 9)
    net.set_normalization(np.zeros(8), np.full(8, 50.0), np.zeros(2), np.full(2, 5.0))
    for mode, val in ((gpu.DT_CFL, 0.4), (gpu.DT_FIXED, 1e-3)):
        a = gpu.Context(cp, prec)
        b = gpu.Context(cp, prec)
        for c in (a, b):
            c.set_state(ps, vz)
            c.set_forcing(fp, fz)
            c.set_time(0.0)
        x = torch.empty((1, n, n, 8), dtype=torch.float32, device="cuda")
        t = torch.empty((1, n, n, 2), dtype=torch.float32, device="cuda")
        for s in range(6):
            if s % 2 == 0:
                closure_inputs(a, x[0])
                net.forward(x, 1, t)
                set_tendency(a, t[0])
            ta, _ = a.advance(1, mode, val)
        set_tendency(a, None)
        tb, _ = closure_advance(b, net, 4, mode, val, every=2)
        tb, _ = closure_advance(b, net, 2, mode, val, every=2)
        assert ta == tb
        for u, v in zip(a.get_state(), b.get_state()):
            np.testing.assert_array_equal(u, v)
    with pytest.raises(gpu.R2D3CError):
        closure_advance(b, net, 3, gpu.DT_FIXED, 1e-3, every=2)


@pytest.mark.parametrize("prec,band", [(0, False), (1, False), (1, True)])
def test_overlapped_les_steps_equal_the_lagged_step_by_step_loop(gpu, prec, band):
    """r2d3c_closure_advance_overlapped (the network for the next step on a
    second stream beside the current step, inside one captured graph): the
    first step of a call takes the tendencies of its own state, step s > 0
    those of the state before step s - 1.  Bit-identical to that schedule
    made one call at a time, in both dt modes, with and without per-shell
    weights (applied to the next tendencies after the join)."""
    import torch
    from rot2d3c_gb300.closure import CNN, closure_advance, closure_inputs, set_band, set_tendency
    n = 32
    _, cp = params(n, omega=1.0, nu=2e-3, nuv=2e-3, hnu=0.1, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 71, amp=20.0)
    fp, fz = random_forcing(g, 72, 2.0, 4.0)
    net = CNN(n, n, 1, 13)
    net.set_normalization(np.zeros(8), np.full(8, 50.0), np.zeros(2), np.full(2, 5.0))
    for mode, val in ((gpu.DT_CFL, 0.4), (gpu.DT_FIXED, 1e-3)):
        a = gpu.Context(cp, prec)
        b = gpu.Context(cp, prec)
        for c in (a, b):
            c.set_state(ps, vz)
            c.set_forcing(fp, fz)
            c.set_time(0.0)
            if band:
                set_band(c, np.linspace(1.0, 0.2, 2 * 12, dtype=np.float32).reshape(2, 12))
        x = torch.empty((1, n, n, 8), dtype=torch.float32, device="cuda")
        t = torch.empty((1, n, n, 2), dtype=torch.float32, device="cuda")
        tn = torch.empty_like(t)
        for nsteps in (3, 2):  # two calls: each starts from its own state's tendencies
            closure_inputs(a, x[0])
            net.forward(x, 1, t)
            for _ in range(nsteps):
                closure_inputs(a, x[0])
                net.forward(x, 1, tn)
                set_tendency(a, t[0])
                ta, _ = a.advance(1, mode, val)
                t.copy_(tn)
        set_tendency(a, None)
        tb, _ = closure_advance(b, net, 3, mode, val, overlap=True)
        tb, _ = closure_advance(b, net, 2, mode, val, overlap=True)
        assert ta == tb
        for u, v in zip(a.get_state(), b.get_state()):
            np.testing.assert_array_equal(u, v)
        # plain steps afterwards: the tendencies are off on both
        a.advance(2, mode, val)
        b.advance(2, mode, val)
        for u, v in zip(a.get_state(), b.get_state()):
            np.testing.assert_array_equal(u, v)
    with pytest.raises(ValueError):
        closure_advance(b, net, 2, gpu.DT_FIXED, 1e-3, every=2, overlap=True)
