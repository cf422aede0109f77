"""Batched ensembles (r2d3c_ensemble_*): every run of a batched, graph-replayed
ensemble equals the same run advanced alone, for both precisions and both
time-step modes; per-run diagnostics equal the single-run ones."""
import numpy as np
import pytest

from tests._helpers import params, random_forcing, random_state

pytestmark = pytest.mark.gpu


def _runs():
    spec = []
    for i, (n, om, nu) in enumerate([(32, 0.1, 2e-3), (32, 3.0, 1e-3), (32, 30.0, 5e-4),
                                     (64, 1.0, 1e-3), (64, 10.0, 2e-4)]):
        _, cp = params(n, omega=om, nu=nu, nuv=nu, hnu=0.1, hnuv=0.1, iflow=0)
        g, ps, vz = random_state(n, 100 + i, kmax_shell=min(10, n // 3), amp=10.0)
        fp, fz = random_forcing(g, 200 + i, 2.0, 4.0)
        spec.append((n, cp, ps, vz, fp, fz))
    return spec


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("mode,val", [(1, 1e-3), (0, 0.3)])
def test_ensemble_runs_equal_single_runs(gpu, prec, mode, val):
    spec = _runs()
    groups = [(32, [s[1] for s in spec[:3]]), (64, [s[1] for s in spec[3:]])]
    ens = gpu.Ensemble(groups, prec)
    for r, (n, cp, ps, vz, fp, fz) in enumerate(spec):
        ens.set_state(r, ps, vz)
        ens.set_forcing(r, fp, fz)
        ens.set_time(r, 0.0)
    times = ens.advance(4, mode, val)
    times = ens.advance(3, mode, val)
    assert ens.kernel_launches() > 0
    plans = ens.plan_report()
    assert [(p["n"], p["runs"]) for p in plans] == [(32, 3), (64, 2)]
    assert all(p["plan"]["pass_a"] and p["plan"]["groups_a"] >= 1 for p in plans)
    for r, (n, cp, ps, vz, fp, fz) in enumerate(spec):
        c = gpu.Context(cp, prec)
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        t, _ = c.advance(4, mode, val)
        t, _ = c.advance(3, mode, val)
        a, b = c.get_state()
        ea, eb = ens.get_state(r)
        np.testing.assert_array_equal(ea, a)
        np.testing.assert_array_equal(eb, b)
        assert times[r] == t
        np.testing.assert_array_equal(ens.cond_check(r, t), c.cond_check(t))
        np.testing.assert_array_equal(ens.spectrum(r)[0], c.spectrum()[0])


def test_ensemble_rejects_mismatched_sizes(gpu):
    _, cp = params(32)
    with pytest.raises(gpu.R2D3CError):
        gpu.Ensemble([(64, [cp])], 0)
