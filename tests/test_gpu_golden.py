"""The CUDA path against the committed golden fixtures (n = 32)."""
import os

import numpy as np
import pytest

from tests._helpers import params, rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_n32.npz")


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
def test_steps_against_golden(gpu, prec, tol):
    d = np.load(GOLD)
    _, cp = params(32, omega=1.0, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, nn=1, mm=2, iflow=0)
    c = gpu.Context(cp, prec)
    c.set_state(d["ps0"], d["vz0"])
    c.set_forcing(d["fp"], d["fz"])
    c.step(1e-3)
    a, b = c.get_state()
    assert rel_l2(a, d["ps1"]) < tol and rel_l2(b, d["vz1"]) < tol
    c.advance(9, gpu.DT_FIXED, 1e-3)
    a, b = c.get_state()
    assert rel_l2(a, d["ps10"]) < tol and rel_l2(b, d["vz10"]) < tol
    cc = c.cond_check(10 * 1e-3)
    ref = d["cond_check10"]
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    assert np.all(np.abs(cc - ref) <= 10 * tol * scale)
    ek, ezk = c.spectrum()
    assert rel_l2(ek, d["ek10"]) < 10 * tol and rel_l2(ezk, d["ezk10"]) < 10 * tol
    f0, f1, f2 = c.transfers()
    for a_, b_ in ((f0, d["fl0_10"]), (f1, d["fl1_10"]), (f2, d["fl2_10"])):
        assert np.abs(a_ - b_).max() <= 100 * tol * np.abs(b_).max()


def test_initial_condition_against_golden(gpu):
    d = np.load(GOLD)
    _, cp = params(32, kup=3.0, u0=0.3, v0=0.2)
    c = gpu.Context(cp, 0)
    s = [5]
    c.initial_conditions(s)
    a, b = c.get_state()
    assert s[0] == int(d["ic_seed_final"][0])
    assert rel_l2(a, d["ic_ps"]) < 1e-12 and rel_l2(b, d["ic_vz"]) < 1e-12
