"""The learned-closure workflow end to end on small grids: DNS snapshots,
CNN training, LES against the filtered DNS.  Checks that every stage runs
through the CUDA library and produces finite, consistent results; the
numbers of the full-size experiment come from ``bench.py --closure``."""
import math

import numpy as np
import pytest


@pytest.mark.gpu
def test_les_workflow_small(gpu):
    from rot2d3c_gb300.les import run_experiment

    r = run_experiment(nf=128, nc=32, nu=2e-3, nsnap=24, snap_every=2, spinup=40, train_steps=40, batch=4,
                       les_steps=120, spec_every=10)
    tr = r["training"]
    assert math.isfinite(tr["loss_first"]) and math.isfinite(tr["loss_last"])
    # standardised targets: the untrained loss is O(1), training lowers it
    assert tr["loss_last"] < tr["loss_first"]
    assert r["dns"]["physical_time"] > 0 and r["dns"]["steps_compared"] > 0
    assert r["les"]["gpu_s"] > 0 and r["dns"]["gpu_s"] > 0
    for name in ("les", "plain", "fallback"):
        e = r["spectrum_error"][name]
        assert all(math.isfinite(v) for v in e.values()), (name, e)
    # a network without held-out skill is not applied: its LES is the fallback
    assert r["les"]["network_applied"] == (tr["val_loss"] < 0.9)
    if not r["les"]["network_applied"]:
        assert r["spectrum_error"]["les"] == r["spectrum_error"]["fallback"]


# A small case of the closure experiment: 512^2 DNS (nu = 1e-4, Omega = 1,
# hypoviscosity 1 with mm = 2, forcing shell 4-6), 400 snapshots filtered to
# 128^2 (k_c = 42), 2000 Adam steps, four 3000-step coarse runs per model
# from held-out snapshots.
GAIN_CASE = dict(nf=512, nc=128, omega=1.0, nu=1e-4, hnu=1.0, nsnap=400, snap_every=10, spinup=3000,
                 train_steps=2000, batch=32, lr=5e-4, les_steps=3000, cfl=0.5, seed=1, starts=4)


@pytest.mark.gpu
def test_trained_closure_beats_the_plain_and_hyperviscous_coarse_runs(gpu):
    """What the trained network gains: the LES (network tendencies on the
    shells next to the cutoff) is closer to the filtered DNS than both the
    plain coarse solver and the hyperviscous fallback on every energy-spectrum
    measure up to k_c (energy-weighted, shape, top third of the shells, worst
    shell), and its energy flux is better than the plain run's and within 5%
    of the fallback's."""
    from rot2d3c_gb300.les import run_experiment

    r = run_experiment(**GAIN_CASE)
    e = r["spectrum_error"]
    print({k: {m: round(v, 3) for m, v in d.items()} for k, d in e.items()})
    for m in ("rel_l1", "mean_abs_log10", "rel_l1_top_third", "max_shell_rel"):
        assert e["les"][m] < e["plain"][m] and e["les"][m] < e["fallback"][m], (m, e)
    assert e["les"]["flux_rel_l1"] < e["plain"]["flux_rel_l1"]
    assert e["les"]["flux_rel_l1"] < 1.05 * e["fallback"]["flux_rel_l1"]


def test_coarse_forcing_is_the_same_physical_field():
    """The coarse copy of the forcing, transformed to physical space, equals
    the fine forcing sampled on every (nf/nc)-th grid point (all its modes are
    resolved on both grids)."""
    from rot2d3c_gb300.les import coarse_forcing, _setup_run

    nf, nc = 64, 16
    _, _, fp, fz = _setup_run(nf, 3)
    cfp, cfz = coarse_forcing(fp, fz, nf, nc)
    for f, c in ((fp, cfp), (fz, cfz)):
        rf = np.fft.irfft2(f.T, s=(nf, nf))
        rc = np.fft.irfft2(c.T, s=(nc, nc))
        np.testing.assert_allclose(rc, rf[:: nf // nc, :: nf // nc], rtol=0, atol=1e-12 * np.abs(rf).max())
