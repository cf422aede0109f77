"""The main-program driver (Rot2D3C.para.f90:2-639 on one GPU) against an
oracle restatement of the same loop: output cadence, file formats, seeds,
CFL time steps and the final state."""
import math
import os
import shutil

import numpy as np
import pytest

from oracle import rot2d3c_oracle as O
from rot2d3c_gb300 import io as fio
from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _oracle_run(n, prm):
    """The reference main loop (stat == 0) with the oracle's routines."""
    p = O.Params(n=n, **{k: v for k, v in prm.items() if k not in ("idir", "odir")})
    g = O.Grid(n)
    seed = [p.seed]
    ps, vz = O.initial_conditions(g, p, seed)
    fp, fz = O.forcing_iflow1(g, p)
    timet, timec, times = p.tstep, p.cstep, p.sstep
    time = 0.0
    bal, spec, fields = [], [], []
    for t in range(1, p.step + 1):
        dt = O.cfl_condition(g, p, ps, vz)
        if timec == p.cstep:
            timec = 0
            bal.append(O.cond_check(g, p, ps, vz, fp, fz, time))
        if times == p.sstep:
            times = 0
            spec.append(O.spectrum(g, ps, vz))
        if timet == p.tstep:
            timet = 0
            fields.append(O.c2r(g, ps / n**2))
        timet += 1
        times += 1
        timec += 1
        time += dt
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, dt)
    return ps, vz, time, bal, spec, fields


def test_driver_matches_oracle_main_loop(gpu, tmp_path):
    from rot2d3c_gb300.driver import Run
    n = 32
    shutil.copy(os.path.join(GOLD, "parameter_small.inp"), tmp_path / "parameter.inp")
    shutil.copy(os.path.join(GOLD, "status_small.inp"), tmp_path / "status.inp")
    os.makedirs(tmp_path / "ins")
    os.makedirs(tmp_path / "outs")
    r = Run(n, str(tmp_path))
    r.setup()
    t_end = r.loop()
    prm = fio.read_parameter_inp(str(tmp_path / "parameter.inp"))
    ops, ovz, otime, bal, spec, fields = _oracle_run(n, prm)
    gps, gvz = r.ctx.get_state()
    assert rel_l2(gps, ops) < 1e-12 and rel_l2(gvz, ovz) < 1e-12
    assert math.isclose(t_end, otime, rel_tol=1e-12)
    got = np.loadtxt(tmp_path / "energy_bal.txt", ndmin=2)
    ref = np.array([b[:12] for b in bal])
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-14)
    assert len(open(tmp_path / "energy_bal.txt").readline()) == 12 * 23 + 1
    for name, sl in (("enstrophy_bal.txt", slice(12, 17)), ("helicity_bal.txt", slice(17, 25)),
                     ("max_min.txt", slice(25, 30))):
        np.testing.assert_allclose(np.loadtxt(tmp_path / name, ndmin=2), np.array([b[sl] for b in bal]),
                                   rtol=1e-10, atol=1e-13)
    for i, (ek, ezk) in enumerate(spec):
        s = np.loadtxt(tmp_path / "outs" / f"spectrum.000{i + 1}.txt")
        np.testing.assert_allclose(s[:, 0], ek, rtol=1e-11, atol=1e-14 * ek.max())
        np.testing.assert_allclose(s[:, 1], ezk, rtol=1e-11, atol=1e-14 * ezk.max())
        assert os.path.exists(tmp_path / "outs" / f"fluxes.000{i + 1}.txt")
    for i, f in enumerate(fields):
        got = fio.read_field(str(tmp_path / "outs" / f"ps.000.00{i + 1}.out"), n)
        assert rel_l2(got, f) < 1e-12
    ts = open(tmp_path / "time_spec.txt").read().split("\n")[0]
    assert ts.startswith("0001") and len(ts) == 16


def test_driver_restart_reads_binary_fields(gpu, tmp_path):
    """stat > 0 (Rot2D3C.para.f90:300-338): the fields of output `stat` are read
    from idir and the output counters resume from it."""
    from rot2d3c_gb300.driver import Run
    n = 32
    lines = open(os.path.join(GOLD, "parameter_small.inp")).read().splitlines()
    lines[1] = "  9                   % 2  step"
    (tmp_path / "parameter.inp").write_text("\n".join(lines) + "\n")
    fio.write_status_inp(str(tmp_path / "status.inp"), 2, 0.5)
    os.makedirs(tmp_path / "ins")
    os.makedirs(tmp_path / "outs")
    rng = np.random.default_rng(3)
    g = O.Grid(n)
    r1 = O.c2r(g, O.random_phase_field(g, 1, 6, -2.0, rng)) * 1e-3
    r2 = O.c2r(g, O.random_phase_field(g, 1, 6, -1.0, rng)) * 1e-3
    fio.write_field(str(tmp_path / "ins" / "ps.000.002.out"), r1)
    fio.write_field(str(tmp_path / "ins" / "vz.000.002.out"), r2)
    r = Run(n, str(tmp_path))
    r.setup()
    assert r.ini == 4 and (chr(r.ic), chr(r.id), chr(r.iu)) == ("0", "0", "2")
    a, b = r.ctx.get_state()
    assert rel_l2(a, O.r2c(g, r1)) < 1e-13 and rel_l2(b, O.r2c(g, r2)) < 1e-13
    r.loop(max_steps=5)   # steps 4..8: timet reaches tstep = 4 at step 8 -> output 003
    assert os.path.exists(tmp_path / "outs" / "ps.000.003.out")
