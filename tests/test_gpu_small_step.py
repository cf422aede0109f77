"""The single-cluster step of small grids (k_step_small: the twelve passes
of an RK4 step in one thread-block cluster launch) against the separate
pass launches: bit-identical states and times in both dt modes, with and
without the learned tendencies, and the autotuner's report of it."""
import numpy as np
import pytest

from tests._helpers import params, random_forcing, random_state

pytestmark = pytest.mark.gpu


def _run(gpu, monkeypatch, small, n, prec, tendency=None):
    import torch
    from rot2d3c_gb300.closure import set_tendency
    monkeypatch.setenv("R2D3C_SMALL", "1" if small else "0")
    _, cp = params(n, omega=1.0, nu=1e-3, nuv=1e-3, hnu=0.1, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 61, amp=10.0)
    fp, fz = random_forcing(g, 62, 2.0, 4.0)
    c = gpu.Context(cp, prec)
    rep = c.plan_report()["small_step"]
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.set_time(0.0)
    if tendency is not None:
        set_tendency(c, torch.from_numpy(tendency).cuda())
    t1, _ = c.advance(4, gpu.DT_CFL, 0.4)
    c.step(2e-3)
    t2, dt2 = c.advance(3, gpu.DT_FIXED, 1e-3)
    if tendency is not None:
        set_tendency(c, None)
    out = c.get_state()
    c.destroy()
    return out, (t1, t2, dt2), rep


@pytest.mark.parametrize("n,prec", [(32, 1), (64, 1), (256, 1), (512, 1), (64, 0), (256, 0)])
def test_small_step_equals_separate_passes(gpu, monkeypatch, n, prec):
    a, ta, rep_a = _run(gpu, monkeypatch, True, n, prec)
    b, tb, rep_b = _run(gpu, monkeypatch, False, n, prec)
    assert rep_a["available"] and rep_a["chosen"] and not rep_b["chosen"]
    assert rep_a["cluster"] in (8, 16) and rep_a["us_cluster"] > 0 and rep_a["us_separate"] > 0
    assert ta == tb
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_small_step_with_tendencies(gpu, monkeypatch):
    n = 128
    rng = np.random.default_rng(5)
    t = (rng.standard_normal((n, n, 2)) * 1e-2).astype(np.float32)
    a, ta, _ = _run(gpu, monkeypatch, True, n, 1, t)
    b, tb, _ = _run(gpu, monkeypatch, False, n, 1, t)
    assert ta == tb
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_large_grids_and_ensembles_keep_separate_passes(gpu, monkeypatch):
    monkeypatch.delenv("R2D3C_SMALL", raising=False)
    rep = gpu.Context(params(1024, iflow=0)[1], 1).plan_report()["small_step"]
    assert not rep["available"] and not rep["chosen"]
