"""Host-side logic of the closure experiment (no GPU): the spectrum error
measures, the band rules of the LES tendencies, the shell rule the device
kernels use against the reference's, and the DNS forcing on the coarse
grid."""
import math

import numpy as np
import pytest

from rot2d3c_gb300 import les
from rot2d3c_gb300.closure import shell_index


def test_spectrum_errors_on_known_spectra():
    kc = 10
    ref = np.concatenate([[0.0], np.linspace(1.0, 0.1, 20)])
    flr = np.linspace(-1.0, 1.0, 21)
    same = les.spectrum_errors(ref, ref, flr, flr, kc)
    assert all(v == 0.0 for v in same.values())
    double = les.spectrum_errors(2 * ref, ref, 2 * flr, flr, kc)
    assert double["rel_l1"] == pytest.approx(1.0)
    assert double["mean_abs_log10"] == pytest.approx(math.log10(2.0))
    assert double["rel_l1_top_third"] == pytest.approx(1.0)
    assert double["max_shell_rel"] == pytest.approx(1.0)
    assert double["flux_rel_l1"] == pytest.approx(1.0)
    # only shells 1 <= k < kc count: a change outside them changes nothing
    off = ref.copy()
    off[0] = 5.0
    off[kc:] *= 3.0
    assert les.spectrum_errors(off, ref, flr, flr, kc)["rel_l1"] == 0.0


def test_band_rules():
    kc, nb = 85, 129
    w = les.band_weights("near_cutoff", kc, nb)
    assert w.shape == (2, nb) and w.dtype == np.float32
    ones = np.flatnonzero(w[0])
    assert ones[0] == 2 * kc // 3 and ones[-1] == kc and len(ones) == kc - 2 * kc // 3 + 1
    np.testing.assert_array_equal(w[0], w[1])
    h = les.band_weights(("high", 10), kc, nb)
    assert np.flatnonzero(h[1])[0] == 10 and np.flatnonzero(h[1])[-1] == kc
    assert les.band_weights(None, kc, nb) is None
    lsq = np.full((2, nb), 0.5, np.float32)
    assert les.band_weights("lsq", kc, nb, lsq) is lsq
    with pytest.raises(ValueError):
        les.band_weights("bogus", kc, nb)


def test_device_shell_rule_equals_the_reference_rule():
    """The kernels that weight tendencies per shell take the shell as
    b = (isqrt(4 ka2) + 1) / 2 in integers, i.e. (2b-1)^2 < 4 ka2 < (2b+1)^2;
    the reference bins by kmn = int(sqrt(ka2) + .5)
    (pseudospec2D_Rot2D3C.f90:615-712).  They agree for every ka2 up to
    2e5 and every 997th up to the largest of an 8192^2 grid, and
    shell_index (the host's map of a plane) is the same rule."""
    ka2 = np.arange(0, 2 * 4096 * 4096 + 1, 997, dtype=np.int64)
    ka2 = np.concatenate([ka2, np.arange(0, 200000, dtype=np.int64)])
    dev = (np.array([math.isqrt(int(4 * k)) for k in ka2]) + 1) // 2
    ref = np.floor(np.sqrt(ka2.astype(np.float64)) + 0.5).astype(np.int64)
    np.testing.assert_array_equal(dev, ref)
    n = 32
    s = shell_index(n)
    h = n // 2
    for i in range(h + 1):
        for j in range(n):
            ky = j if j < h else j - n
            assert s[i, j] == (math.isqrt(4 * (i * i + ky * ky)) + 1) // 2


def test_coarse_forcing_keeps_the_retained_modes():
    """A forcing mode of the fine grid inside the coarse grid's half-plane
    lands on the same (kx, ky) of the coarse grid, scaled by (nc/nf)^2
    (the transforms are unnormalised)."""
    nf, nc = 64, 16
    fp = np.zeros((nf // 2 + 1, nf), np.complex128)
    fz = np.zeros_like(fp)
    fp[3, 2] = 1.0 + 2.0j       # (kx, ky) = (3, 2)
    fz[2, nf - 5] = -0.5j       # (kx, ky) = (2, -5)
    cp, cz = les.coarse_forcing(fp, fz, nf, nc)
    s = (nc / nf) ** 2
    assert cp.shape == (nc // 2 + 1, nc)
    assert cp[3, 2] == pytest.approx((1.0 + 2.0j) * s)
    assert cz[2, nc - 5] == pytest.approx(-0.5j * s)
    assert np.count_nonzero(cp) == 1 and np.count_nonzero(cz) == 1
