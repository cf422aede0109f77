"""The RK step (Rot2D3C.para.f90:545-611) and the graph-replayed main loop
against the oracle; analytic known answers for its linear part."""
import math

import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import params, random_forcing, random_state, rel_l2

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 1e-5}


def _run_oracle(g, p, ps, vz, fp, fz, dt, nsteps):
    for _ in range(nsteps):
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, dt)
    return ps, vz


@pytest.mark.parametrize("n", [16, 32, 64])
@pytest.mark.parametrize("omega", [0.0, 1.0])
@pytest.mark.parametrize("prec", [0, 1])
def test_one_step_matches_oracle(gpu, n, omega, prec):
    p, cp = params(n, omega=omega, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 11)
    fp, fz = random_forcing(g, 12, 2.0, 4.0)
    dt = 1e-3
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.step(dt)
    gps, gvz = c.get_state()
    ops, ovz = _run_oracle(g, p, ps, vz, fp, fz, dt, 1)
    assert rel_l2(gps, ops) < TOL[prec]
    assert rel_l2(gvz, ovz) < TOL[prec]


@pytest.mark.parametrize("prec", [0, 1])
def test_ten_steps_match_oracle(gpu, prec):
    n = 64
    p, cp = params(n, omega=1.0, nu=1e-3, hnu=0.1, nuv=1e-3, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 21, amp=50.0)
    fp, fz = random_forcing(g, 22)
    dt = 1e-3
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    for _ in range(10):
        c.step(dt)
    gps, gvz = c.get_state()
    ops, ovz = _run_oracle(g, p, ps, vz, fp, fz, dt, 10)
    assert rel_l2(gps, ops) < TOL[prec]
    assert rel_l2(gvz, ovz) < TOL[prec]


def test_untruncated_state_is_truncated_by_the_step(gpu):
    """A restart state with content outside the 2/3 mask (set_state / the
    restart R2C does not truncate) comes out of one step exactly as the
    reference's truncating update leaves it."""
    n = 32
    p, cp = params(n, omega=0.5, iflow=0)
    g = O.Grid(n)
    rng = np.random.default_rng(5)
    r1, r2 = rng.standard_normal((n, n)), rng.standard_normal((n, n))
    ps, vz = O.r2c(g, r1) / n**2, O.r2c(g, r2) / n**2
    fp, fz = random_forcing(g, 6)
    c = gpu.Context(cp, 0)
    c.set_state_physical(r1 / n**2, r2 / n**2)
    c.set_forcing(fp, fz)
    c.step(1e-3)
    gps, gvz = c.get_state()
    ops, ovz = _run_oracle(g, p, ps, vz, fp, fz, 1e-3, 1)
    assert rel_l2(gps, ops) < 1e-12 and rel_l2(gvz, ovz) < 1e-12
    mask = g.ka2 > g.kmax
    assert np.all(gps[mask] == 0) and np.all(gvz[mask] == 0)


@pytest.mark.parametrize("prec", [0, 1])
def test_graph_advance_equals_repeated_steps(gpu, prec):
    n = 64
    _, cp = params(n, omega=2.0, iflow=0)
    g, ps, vz = random_state(n, 31, amp=20.0)
    fp, fz = random_forcing(g, 32)
    a = gpu.Context(cp, prec)
    b = gpu.Context(cp, prec)
    for c in (a, b):
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
    for _ in range(5):
        a.step(2e-3)
    t, dtl = b.advance(5, gpu.DT_FIXED, 2e-3)
    np.testing.assert_array_equal(a.get_state()[0], b.get_state()[0])
    np.testing.assert_array_equal(a.get_state()[1], b.get_state()[1])
    assert dtl == 2e-3 and abs(t - 5 * 2e-3) < 1e-15


@pytest.mark.parametrize("prec", [0, 1])
def test_cfl_advance_matches_oracle_loop(gpu, prec):
    """Main loop with CFL time steps (Rot2D3C.para.f90:399, :537, :545-611)."""
    n = 32
    p, cp = params(n, omega=1.0, cfl=0.3, iflow=0)
    g, ps, vz = random_state(n, 41, amp=30.0)
    fp, fz = random_forcing(g, 42)
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.set_time(0.0)
    t, dtl = c.advance(6, gpu.DT_CFL, p.cfl)
    time = 0.0
    for _ in range(6):
        dt = O.cfl_condition(g, p, ps, vz)
        time += dt
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, dt)
    gps, gvz = c.get_state()
    tol = {0: 1e-12, 1: 1e-5}[prec]
    assert rel_l2(gps, ps) < tol and rel_l2(gvz, vz) < tol
    assert abs(t - time) <= tol * time and abs(dtl - dt) <= tol * dt


def test_cfl_matches_oracle(gpu):
    n = 64
    p, cp = params(n, omega=3.0, cfl=0.5, nu=2e-3, nn=2, nuv=1e-3, nnv=1)
    g, ps, vz = random_state(n, 51, amp=10.0)
    c = gpu.Context(cp, 0)
    c.set_state(ps, vz)
    assert abs(c.CFL_condition(p.cfl) - O.cfl_condition(g, p, ps, vz)) < 1e-14 * O.cfl_condition(g, p, ps, vz)


@pytest.mark.parametrize("nn,mm", [(1, 2), (2, 1), (3, 0)])
def test_linear_decay_known_answer(gpu, nn, mm):
    """With one Fourier mode the brackets vanish and the scheme reduces to
    psi1 = psi0/(1 + dt (nu k^2nn + hnu k^-2mm)) (Rot2D3C.para.f90:585-592)."""
    n = 32
    nu, hnu, dt = 2e-3, 0.3, 5e-3
    _, cp = params(n, omega=0.0, nu=nu, hnu=hnu, nn=nn, mm=mm, nuv=nu, hnuv=hnu, nnv=nn, mmv=mm, iflow=0)
    g = O.Grid(n)
    ps = np.zeros(g.shape_spec, complex)
    vz = np.zeros(g.shape_spec, complex)
    ps[3, 4] = 2.0 + 1.0j
    vz[3, 4] = -1.0 + 0.5j
    c = gpu.Context(cp, 0)
    c.set_state(ps, vz)
    c.set_forcing(np.zeros_like(ps), np.zeros_like(ps))
    c.step(dt)
    gps, gvz = c.get_state()
    k2 = 25.0
    fac = 1.0 / (1.0 + dt * (nu * k2**nn + hnu * k2 ** (-mm)))
    assert abs(gps[3, 4] - ps[3, 4] * fac) < 1e-15
    assert abs(gvz[3, 4] - vz[3, 4] * fac) < 1e-15
    gps[3, 4] = 0
    assert np.abs(gps).max() < 1e-15


def test_coriolis_known_answer(gpu):
    """One mode, no dissipation: d psi/dt = 2 Omega i ky vz / k^2,
    d vz/dt = 2 Omega i ky psi.  Low-storage RK of order 4 gives the 4th-order
    Taylor polynomial of exp(dt A)."""
    n = 32
    omega, dt = 3.0, 0.02
    _, cp = params(n, omega=omega, nu=0.0, hnu=0.0, nuv=0.0, hnuv=0.0, iflow=0)
    g = O.Grid(n)
    ps = np.zeros(g.shape_spec, complex)
    vz = np.zeros(g.shape_spec, complex)
    kx, ky = 2, 5
    ps[kx, ky] = 0.7 - 0.2j
    vz[kx, ky] = 0.1 + 0.4j
    c = gpu.Context(cp, 0)
    c.set_state(ps, vz)
    c.set_forcing(np.zeros_like(ps), np.zeros_like(ps))
    c.step(dt)
    gps, gvz = c.get_state()
    k2 = kx * kx + ky * ky
    A = np.array([[0, 2 * omega * 1j * ky / k2], [2 * omega * 1j * ky, 0]])
    M = sum(np.linalg.matrix_power(dt * A, k) / math.factorial(k) for k in range(5))
    y = M @ np.array([ps[kx, ky], vz[kx, ky]])
    assert abs(gps[kx, ky] - y[0]) < 1e-15 and abs(gvz[kx, ky] - y[1]) < 1e-15
