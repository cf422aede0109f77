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
