"""Diagnostic reductions (cond_check, spectrum, transfers) and field outputs
against the oracle (pseudospec2D_Rot2D3C.f90:455-837, Rot2D3C.para.f90:476-519)."""
import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import params, random_forcing, random_state, rel_l2

pytestmark = pytest.mark.gpu


def _setup(gpu, n, prec, **kw):
    p, cp = params(n, **kw)
    g, ps, vz = random_state(n, 61, amp=3.0)
    fp, fz = random_forcing(g, 62, 3.0, 5.0)
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    return p, g, c, ps, vz, fp, fz


@pytest.mark.parametrize("prec", [0, 1])
def test_cond_check(gpu, prec):
    p, g, c, ps, vz, fp, fz = _setup(gpu, 64, prec, omega=1.5, kup=4.0, nn=2, mm=1, nnv=1, mmv=2,
                                     nu=1e-3, hnu=0.2, nuv=2e-3, hnuv=0.1)
    got = c.cond_check(0.25)
    ref = O.cond_check(g, p, ps, vz, fp, fz, 0.25)
    rtol = 1e-12 if prec == 0 else 2e-6
    # scale per quantity: the bigger of |ref| and the energy it is built from
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    assert np.all(np.abs(got - ref) <= rtol * scale), np.c_[got, ref]


@pytest.mark.parametrize("prec", [0, 1])
def test_spectrum_and_transfers(gpu, prec):
    p, g, c, ps, vz, fp, fz = _setup(gpu, 64, prec)
    ek, ezk = c.spectrum()
    oek, oezk = O.spectrum(g, ps, vz)
    tol = 1e-12 if prec == 0 else 2e-6
    assert rel_l2(ek, oek) < tol and rel_l2(ezk, oezk) < tol
    f0, f1, f2 = c.transfers()
    o0, o1, o2 = O.transfers(g, ps, vz)
    tol = 1e-11 if prec == 0 else 2e-5
    for a, b in ((f0, o0), (f1, o1), (f2, o2)):
        assert np.abs(a - b).max() <= tol * np.abs(b).max()
    # the nonlinear transfers conserve energy: the total flux is ~0
    assert abs(f1.sum()) < 1e-9 * np.abs(f1).max() * len(f1) or prec == 1


@pytest.mark.parametrize("prec", [0, 1])
def test_field_outputs(gpu, prec):
    p, g, c, ps, vz, fp, fz = _setup(gpu, 32, prec)
    n = 32
    tmp = 1.0 / n**2
    refs = {
        gpu.FIELD_PS: O.c2r(g, ps * tmp),
        gpu.FIELD_VZ: O.c2r(g, vz * tmp),
        gpu.FIELD_WW: O.c2r(g, ps * g.ka2 * tmp),
        gpu.FIELD_INVLAP_PSI: O.c2r(g, O.inv_laplak2(g, ps) * tmp),
    }
    tol = 1e-13 if prec == 0 else 2e-6
    for w, ref in refs.items():
        assert rel_l2(c.get_field(w), ref) < tol


def test_reductions_are_deterministic(gpu):
    p, g, c, ps, vz, fp, fz = _setup(gpu, 128, 0)
    a = c.cond_check(1.0)
    b = c.cond_check(1.0)
    np.testing.assert_array_equal(a, b)
    s1 = c.transfers()
    s2 = c.transfers()
    for x, y in zip(s1, s2):
        np.testing.assert_array_equal(x, y)
