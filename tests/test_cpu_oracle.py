"""The C/OpenMP restatement agrees with the NumPy oracle (two independent
restatements of the reference, cross-checked to ~1e-13)."""
import numpy as np
import pytest

from oracle import cpu_oracle as CO
from oracle import rot2d3c_oracle as O
from tests._helpers import random_forcing, random_state, rel_l2


@pytest.mark.parametrize("n", [16, 64])
def test_transforms(n):
    g = O.Grid(n)
    rng = np.random.default_rng(n)
    r = rng.standard_normal((n, n))
    c = rng.standard_normal((n // 2 + 1, n)) + 1j * rng.standard_normal((n // 2 + 1, n))
    assert rel_l2(CO.r2c(n, r), O.r2c(g, r)) < 1e-14
    assert rel_l2(CO.c2r(n, c), O.c2r(g, c)) < 1e-14


@pytest.mark.parametrize("cfl_mode", [False, True])
def test_steps(cfl_mode):
    n = 32
    p = O.Params(n=n, omega=1.0, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, iflow=0, cfl=0.3)
    g, ps, vz = random_state(n, 9, amp=20.0)
    fp, fz = random_forcing(g, 10)
    a, b, dtl = CO.run(p, ps, vz, fp, fz, 3, p.cfl if cfl_mode else 1e-3, cfl_mode, threads=2)
    for _ in range(3):
        dt = O.cfl_condition(g, p, ps, vz) if cfl_mode else 1e-3
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, dt)
    assert rel_l2(a, ps) < 1e-13 and rel_l2(b, vz) < 1e-13
    assert abs(dtl - dt) < 1e-14 * dt
