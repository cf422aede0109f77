"""Forcing (iflow 1, 2, 3), the seeded initial condition and the seed
bookkeeping of the reference (Rot2D3C.para.f90:245-381,
pseudospec2D_Rot2D3C.f90:977-1126)."""
import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from tests._helpers import params, random_state, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_initial_conditions(gpu, prec):
    n = 32
    p, cp = params(n, kup=3.0, u0=0.3, v0=0.2)
    c = gpu.Context(cp, prec)
    s = [5]
    c.initial_conditions(s)
    so = [5]
    ops, ovz = O.initial_conditions(O.Grid(n), p, so)
    assert s == so
    gps, gvz = c.get_state()
    tol = 1e-12 if prec == 0 else 2e-6
    assert rel_l2(gps, ops) < tol and rel_l2(gvz, ovz) < tol


@pytest.mark.parametrize("prec", [0, 1])
def test_iflow1_forcing(gpu, prec):
    n = 32
    p, cp = params(n, kup=3.0, fp0=0.7, fz0=1.3, iflow=1)
    c = gpu.Context(cp, prec)
    c.forcing_init([1], [2])
    fp, fz = c.get_forcing()
    ofp, ofz = O.forcing_iflow1(O.Grid(n), p)
    tol = 1e-12 if prec == 0 else 2e-6
    assert rel_l2(fp, ofp) < tol and rel_l2(fz, ofz) < tol


def test_rand_force_iflow3(gpu):
    n = 32
    p, cp = params(n, kup=5.0, fp0=0.5, fz0=0.8, iflow=3)
    g = O.Grid(n)
    c = gpu.Context(cp, 0)
    seed, seed1 = [7], [8]
    so, s1o = [7], [8]
    for dt in (1e-3, 2.5e-3, 4e-4):
        c.rand_force(dt, seed, seed1)
        ofp = O.rand_force(g, p.kdn, p.kup, p.fp0, dt, so, 1)
        ofz = O.rand_force(g, p.kdn, p.kup, p.fz0, dt, s1o, 0)
        fp, fz = c.get_forcing()
        np.testing.assert_array_equal(fp, ofp)
        np.testing.assert_array_equal(fz, ofz)
    assert seed == so and seed1 == s1o


def test_iflow3_cfl_loop_matches_oracle(gpu):
    """CFL dt, rand_force each step and the RK step, graph-replayed."""
    n = 32
    p, cp = params(n, kup=4.0, kdn=4.0, fp0=1.0, fz0=1.0, iflow=3, cfl=0.4, omega=0.5)
    g, ps, vz = random_state(n, 71, amp=5.0)
    c = gpu.Context(cp, 0)
    c.set_state(ps, vz)
    c.set_time(0.0)
    seed, seed1 = [3], [4]
    t, dtl = c.advance(5, gpu.DT_CFL, p.cfl, seed, seed1)
    so, s1o = [3], [4]
    fp = fz = np.zeros(g.shape_spec, complex)
    time = 0.0
    for _ in range(5):
        dt = O.cfl_condition(g, p, ps, vz)
        fp = O.rand_force(g, p.kdn, p.kup, p.fp0, dt, so, 1)
        fz = O.rand_force(g, p.kdn, p.kup, p.fz0, dt, s1o, 0)
        time += dt
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, dt)
    gps, gvz = c.get_state()
    assert seed == so and seed1 == s1o
    assert rel_l2(gps, ps) < 1e-12 and rel_l2(gvz, vz) < 1e-12
    assert abs(t - time) < 1e-12 * time


@pytest.mark.parametrize("prec", [0, 1])
def test_const_inj_iflow2_step(gpu, prec):
    n = 32
    p, cp = params(n, kdn=3.0, kup=5.0, fp0=0.5, fz0=0.6, iflow=2, omega=0.3)
    g, ps, vz = random_state(n, 81, amp=2.0)
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    seed, seed1 = [11], [0]
    c.forcing_init(seed, seed1)
    so, s1o = [11], [0]
    from oracle.rot2d3c_oracle import Seeds
    s1o[0] = so[0] + 1
    ofp = O.const_inj(g, ps, p.kdn, p.kup, p.fp0, 1, s1o)
    ofz = O.const_inj(g, vz, p.kdn, p.kup, p.fz0, 0, so)
    fp, fz = c.get_forcing()
    tol = 1e-12 if prec == 0 else 2e-6
    assert rel_l2(fp, ofp) < tol and rel_l2(fz, ofz) < tol
    assert seed == so and seed1 == s1o
    sd = Seeds(seed=so, seed1=s1o)
    for _ in range(2):
        c.step(1e-3, seed, seed1)
        ps, vz, ofp, ofz = O.rk_step(g, p, ps, vz, ofp, ofz, 1e-3, sd)
    gps, gvz = c.get_state()
    tol = 1e-12 if prec == 0 else 1e-5
    assert rel_l2(gps, ps) < tol and rel_l2(gvz, vz) < tol
    fp, fz = c.get_forcing()
    assert rel_l2(fp, ofp) < tol and rel_l2(fz, ofz) < tol
    assert seed == sd.seed and seed1 == sd.seed1
