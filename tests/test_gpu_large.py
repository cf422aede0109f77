"""The FP32 grids that run the pipelined, persistent pass B (n = 2048, 4096)
and the radix-16 transforms: steps against the FP64 path on the same inputs
(the FP64 path matches the oracle to 1e-12 at the sizes the oracle runs
quickly), the CFL time step of the fused maximum, and batched runs against
single runs (bit-exact: every row pair is computed the same way whatever CTA
carries it)."""
import numpy as np
import pytest

from tests._helpers import params, random_forcing, random_state, rel_l2

pytestmark = pytest.mark.gpu


def _case(n, seed):
    _, cp = params(n, omega=2.0, nu=1e-5, nuv=1e-5, hnu=0.1, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, seed, kmax_shell=min(100.0, n / 3.0), slope=-3.0, amp=float(n) ** 2)
    fp, fz = random_forcing(g, seed + 1, 20.0, 22.0)
    return cp, ps, vz, fp, fz


def _advance(gpu, prec, cp, ps, vz, fp, fz, nsteps, mode, val):
    c = gpu.Context(cp, prec)
    c.set_state(ps, vz)
    c.set_forcing(fp, fz)
    c.set_time(0.0)
    t, dt = c.advance(nsteps, mode, val)
    a, b = c.get_state()
    c.destroy()
    return a, b, t, dt


@pytest.mark.parametrize("n", [512, 1024, 2048, 4096])
def test_fp32_cfl_steps_match_fp64(gpu, n):
    cp, ps, vz, fp, fz = _case(n, 7)
    a32, b32, t32, dt32 = _advance(gpu, 1, cp, ps, vz, fp, fz, 3, gpu.DT_CFL, 0.5)
    a64, b64, t64, dt64 = _advance(gpu, 0, cp, ps, vz, fp, fz, 3, gpu.DT_CFL, 0.5)
    assert abs(dt32 - dt64) <= 1e-5 * dt64
    assert abs(t32 - t64) <= 1e-5 * t64
    assert rel_l2(a32, a64) < 1e-5
    assert rel_l2(b32, b64) < 1e-5


@pytest.mark.parametrize("n", [2048, 4096])
def test_fp32_batched_equals_single(gpu, n):
    runs = [_case(n, 30 + 2 * i) for i in range(2)]
    ens = gpu.Ensemble([(n, [r[0] for r in runs])], 1)
    for i, (cp, ps, vz, fp, fz) in enumerate(runs):
        ens.set_state(i, ps, vz)
        ens.set_forcing(i, fp, fz)
        ens.set_time(i, 0.0)
    times = ens.advance(2, gpu.DT_CFL, 0.5)
    for i, (cp, ps, vz, fp, fz) in enumerate(runs):
        a, b, t, _ = _advance(gpu, 1, cp, ps, vz, fp, fz, 2, gpu.DT_CFL, 0.5)
        ea, eb = ens.get_state(i)
        np.testing.assert_array_equal(ea, a)
        np.testing.assert_array_equal(eb, b)
        assert times[i] == t
    ens.destroy()


def test_fp32_vs_fp64_at_8192_spectra(gpu):
    """8192^2, 50 CFL steps (nu = 2e-6, Omega = 1, IC k^-3 on 1 <= |k| <= 200,
    forcing shell 30-32): the FP32 path against the FP64 path, per field and
    per shell of the energy spectrum."""
    n = 8192
    _, cp = params(n, omega=1.0, nu=2e-6, nuv=2e-6, hnu=0.1, hnuv=0.1, iflow=0)
    g, ps, vz = random_state(n, 81, kmax_shell=200.0, slope=-3.0, amp=float(n) ** 2)
    fp, fz = random_forcing(g, 82, 30.0, 32.0)
    out = {}
    for prec in (0, 1):
        c = gpu.Context(cp, prec)
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        c.advance(50, gpu.DT_CFL, 0.5)
        out[prec] = (c.get_state(), c.spectrum()[0])
        c.destroy()
    (a64, b64), ek64 = out[0]
    (a32, b32), ek32 = out[1]
    assert rel_l2(a32, a64) < 2e-5
    assert rel_l2(b32, b64) < 2e-5
    live = ek64 > 1e-12 * ek64.max()
    assert np.max(np.abs(ek32[live] - ek64[live]) / ek64[live]) < 1e-3


@pytest.mark.parametrize("n", [512, 1024, 2048, 4096])
def test_autotuned_pass_b_variants_are_bit_identical(gpu, monkeypatch, n):
    """The plan autotuner times the pass-B launch schedules at context
    creation; both schedules give bit-identical steps, so the choice never
    changes results."""
    cp, ps, vz, fp, fz = _case(n, 11)
    c = gpu.Context(cp, 1)
    rep = c.plan_report()
    variants_b = {r["variant"] for r in rep["pass_b"]}
    assert variants_b == ({"per_row_pair", "persistent", "split"} if n <= 1024 else {"per_row_pair", "persistent"})
    assert rep["pass_a"] and all(r["us"] > 0 for r in rep["pass_a"])
    assert all(r["us"] > 0 for r in rep["pass_b"]) and rep["chosen"] in variants_b
    assert {r["variant"] for r in rep["pass_c"]} == {"per_column_pair", "persistent"}
    assert all(r["us"] > 0 for r in rep["pass_c"]) and rep["chosen_c"] in ("per_column_pair", "persistent")
    c.destroy()
    out = []
    for mb, mc, groups in (("per_row_pair", "per_column_pair", None), ("persistent", "persistent", None),
                           ("persistent", "per_column_pair", None), ("persistent", "per_column_pair", "0,1,0,0,2"),
                           ("split" if n <= 1024 else "persistent", "persistent", None)):
        monkeypatch.setenv("R2D3C_PASSB", mb)
        monkeypatch.setenv("R2D3C_PASSC", mc)
        if groups:
            monkeypatch.setenv("R2D3C_GROUPS", groups)
        else:
            monkeypatch.delenv("R2D3C_GROUPS", raising=False)
        c = gpu.Context(cp, 1)
        assert c.plan_report()["chosen"] == mb and c.plan_report()["chosen_c"] == mc
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        c.advance(2, gpu.DT_CFL, 0.5)
        out.append(c.get_state())
        c.destroy()
    for o in out[1:]:
        for u, v in zip(out[0], o):
            np.testing.assert_array_equal(u, v)
    small = gpu.Context(params(64, iflow=0)[1], 1).plan_report()
    assert {r["variant"] for r in small["pass_b"]} == {"per_row_pair", "split"} and small["chosen"] in (
        "per_row_pair", "split")
    assert {r["variant"] for r in small["pass_c"]} == {"per_column_pair"} and small["chosen_c"] == "per_column_pair"


@pytest.mark.parametrize("n,prec", [(256, 1), (256, 0), (512, 1), (1024, 0)])
def test_launch_shapes_are_bit_identical(gpu, monkeypatch, n, prec):
    """Groups per CTA (passes A, B, C) and pass A's field chunks are launch
    shapes only: every forced choice steps to the same bits as the tuned one."""
    cp, ps, vz, fp, fz = _case(n, 5)
    out, reps = [], []
    for forced in (None, "1,6,1,1", "0,1,0,0", "2,3,1,2", "0,1,0,1,2", "1,2,1,2,2", "split", "0,1,0,0,2,4",
                   "0,1,0,0,2,2"):
        if forced is None:
            monkeypatch.delenv("R2D3C_GROUPS", raising=False)
        elif forced != "split":
            monkeypatch.setenv("R2D3C_GROUPS", forced)
        monkeypatch.setenv("R2D3C_PASSB", "split" if forced == "split" else "per_row_pair")
        monkeypatch.setenv("R2D3C_PASSC", "per_column_pair")
        c = gpu.Context(cp, prec)
        reps.append(c.plan_report())
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        c.advance(3, gpu.DT_CFL, 0.5)
        out.append(c.get_state())
        c.destroy()
    assert reps[1]["groups_a"] == 1 and reps[1]["field_chunks_a"] == 6 and reps[1]["groups_b"] == 1
    assert reps[3]["field_chunks_a"] == 3
    # pass C's C1 and C2 updates split over two CTAs per column pair (FP32)
    assert reps[4]["chunks_c"] == (2 if prec == 1 else 1) and reps[5]["groups_c"] == 2
    assert reps[6]["chosen"] == "split"
    # teams of groups sharing a column pair's RK update (FP32)
    assert reps[7]["team_c"] == (4 if prec == 1 else 1) and reps[8]["team_c"] == (2 if prec == 1 else 1)
    for o in out[1:]:
        for u, v in zip(out[0], o):
            np.testing.assert_array_equal(u, v)
    monkeypatch.setenv("R2D3C_GROUPS", "3,1,1,1")
    with pytest.raises(gpu.R2D3CError):
        gpu.Context(cp, prec)
    monkeypatch.setenv("R2D3C_GROUPS", "0,1,0,0,3")
    with pytest.raises(gpu.R2D3CError):
        gpu.Context(cp, prec)


@pytest.mark.parametrize("n", [1024, 4096])
def test_fp32_pass_a_radices_stay_within_the_fp32_bound(gpu, monkeypatch, n):
    """The plan autotuner may run FP32 pass A with radix 16 or 8 (they round
    differently, like FFTW's measured plans): each radix, forced, steps
    within the FP32 path's bound of the FP64 path, and every engine of one
    precision and n in a process uses the same radix."""
    cp, ps, vz, fp, fz = _case(n, 13)
    a64, b64, _, _ = _advance(gpu, 0, cp, ps, vz, fp, fz, 3, gpu.DT_CFL, 0.5)
    for radix in (16, 8):
        monkeypatch.setenv("R2D3C_RADIX_A", str(radix))
        c = gpu.Context(cp, 1)
        rep = c.plan_report()
        assert rep["radix_a"] == radix and {r["radix"] for r in rep["pass_a"]} == {8, 16}
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        c.advance(3, gpu.DT_CFL, 0.5)
        a, b = c.get_state()
        c.destroy()
        assert rel_l2(a, a64) < 1e-5 and rel_l2(b, b64) < 1e-5, (radix, rel_l2(a, a64), rel_l2(b, b64))
    monkeypatch.delenv("R2D3C_RADIX_A")
    r1 = gpu.Context(cp, 1).plan_report()["radix_a"]
    r2 = gpu.Context(cp, 1).plan_report()["radix_a"]
    assert r1 == r2 and r1 in (8, 16)


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_pass_c_carrying_pass_a_is_bit_identical(gpu, monkeypatch, n):
    """FP32 grids up to 512: inside r2d3c_advance each substep's pass C
    launch also runs the next substep's pass A on the column pairs it has
    just updated (plan_report "fused_ca"; each advance call starts with one
    separate pass A).  With R2D3C_FUSE_CA=0 pass A keeps its own launch.
    The states and times are bit-identical over several calls, in both dt
    modes, with closure tendencies on, under forced pass C shapes (two CTAs
    per column pair, teams of 2 and 4 groups)."""
    import torch
    from rot2d3c_gb300.closure import set_tendency
    cp, ps, vz, fp, fz = _case(n, 17)
    rng = np.random.default_rng(n)
    tend = torch.from_numpy((float(n) * rng.standard_normal((n, n, 2))).astype(np.float32)).cuda()
    shapes = (None, "0,1,0,1,2", "0,1,0,0,2,4", "0,1,0,0,2,2") if n >= 256 else (None,)
    for forced in shapes:
        outs = []
        for fuse in ("1", "0"):
            monkeypatch.setenv("R2D3C_FUSE_CA", fuse)
            monkeypatch.setenv("R2D3C_PASSC", "per_column_pair")
            if forced:
                monkeypatch.setenv("R2D3C_GROUPS", forced)
            else:
                monkeypatch.delenv("R2D3C_GROUPS", raising=False)
            c = gpu.Context(cp, 1)
            assert c.plan_report()["fused_ca"] == (fuse == "1")
            c.set_state(ps, vz)
            c.set_forcing(fp, fz)
            c.set_time(0.0)
            t1, _ = c.advance(3, gpu.DT_CFL, 0.5)
            t2, _ = c.advance(2, gpu.DT_FIXED, 1e-4)
            set_tendency(c, tend)
            t3, _ = c.advance(2, gpu.DT_CFL, 0.5)
            set_tendency(c, None)
            outs.append((c.get_state(), (t1, t2, t3)))
            c.destroy()
        (s1, times1), (s0, times0) = outs
        assert times1 == times0, forced
        for u, v in zip(s1, s0):
            np.testing.assert_array_equal(u, v)
    monkeypatch.setenv("R2D3C_FUSE_CA", "2")
    with pytest.raises(gpu.R2D3CError):
        gpu.Context(cp, 1)
