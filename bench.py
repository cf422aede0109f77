#!/usr/bin/env python
"""Benchmark of the Rot2D3C RK4 time step on GB300.

Workload: a single large run at n = 4096^2, RK order 4, fixed dt = 1e-4,
nu = nuv = 1e-5 (nn = 1), hypoviscosity hnu = hnuv = 0.1 (nabla^-4, mm = 2),
Omega = 10, a seeded random-phase initial spectrum ~ k^-3 for 1 <= |k| <= 100
(energy(ps,1) = energy(vz,0) = 0.5) and a seeded, time-constant random-phase
forcing in the shell 20 <= |k| <= 22 normalised like iflow = 1
(energy(fp,1) = energy(fz,0) = 1).  All inputs are synthetic.

One bench step = one RK4 step.  The headline `value` is the FP64 drop-in
path (the reference's own arithmetic), device-timed over graph-replayed
steps; `e2e` is the same path through the C-ABI with the state coming from
and going back to pinned host FP64 buffers on every step; `e2e_loop` is the
drop-in main loop (CFL time step every step, cond_check / spectrum +
transfers / field output at a fixed cadence) through the C-ABI.  The FP32
path (FP32 fields and transforms with compensated twiddles, FP64
reductions) is reported in `fp32`, with its speed-up over FP64 and the
relative L2 error of omega and vz against the FP64 path and against the
CPU oracle after 100 steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: one field does not shard (replicas only): every rank runs its own
replica and `value` counts the steps of all ranks.  The batched ensemble
leg partitions its runs over the ranks by cost (n^2 log2 n per step) and
gathers the per-run diagnostics on the host.  `--gpus N` without a
torchrun environment re-launches itself under torch.distributed.run with N
ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
import time as time_mod

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK steps/s at 4096^2 FP64 vs FP32 (err vs FP64); batched runs/s; LES-vs-DNS gain"
UNIT = "RK4 steps/s"
WORKLOAD = dict(n=4096, dt=1e-4, nu=1e-5, hnu=0.1, nn=1, mm=2, omega=10.0, ic_kmin=1.0,
                ic_kmax=100.0, ic_slope=-3.0, f_kmin=20.0, f_kmax=22.0, ic_seed=1, f_seed=2)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=WORKLOAD["n"])
    ap.add_argument("--fp32-steps", type=int, default=0, help="timed FP32 steps (default: --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="profiling runs of the FP32 path alone: skip the FP64 legs (the line then reports FP32)")
    ap.add_argument("--err-steps", type=int, default=100)
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--ensemble-steps", type=int, default=500)
    ap.add_argument("--no-closure", action="store_true")
    ap.add_argument("--no-precision-study", action="store_true", help="skip the 8192^2 FP32-vs-FP64 leg")
    ap.add_argument("--closure-full", action="store_true",
                    help="also run the full-size closure experiment: 2048^2 DNS at nu = 5e-6, 2000 snapshots, "
                         "20k Adam steps, 5000 LES steps, Omega 1 and 10 (several minutes)")
    ap.add_argument("--e2e-steps", type=int, default=20, help="steps of the host round-trip e2e leg")
    ap.add_argument("--loop-steps", type=int, default=200, help="steps of the main-loop e2e leg (0: skip)")
    ap.add_argument("--oracle-steps", type=int, default=100,
                    help="CPU oracle steps for the error against the oracle and the CPU baseline (0: skip)")
    ap.add_argument("--closure-small", action="store_true",
                    help="closure leg on a small case (512^2 DNS, 128^2 LES, few steps): for profiling its kernels")
    return ap.parse_args()


# ---------------------------------------------------------------- inputs
def _grid(n):
    import numpy as np
    h = n // 2
    ka = np.concatenate([np.arange(h), np.arange(h) - h]).astype(np.float64)
    kx = ka[: h + 1]
    return ka, kx, kx[:, None] ** 2 + ka[None, :] ** 2


def _energy(a, ka2, kin, n):
    import numpy as np
    two = np.full((a.shape[0], 1), 2.0)
    two[0, 0] = 1.0
    return float(np.sum(two * np.abs(a) ** 2 * ka2 ** kin) / float(n) ** 4)


def synthetic_field(n, kmin, kmax, amp_slope, seed):
    """Random-phase spectral field in [kx][ky] layout with |a(k)| ~ k**amp_slope
    on kmin <= |k| <= kmax; the kx = 0 column is made Hermitian."""
    import numpy as np
    ka, kx, ka2 = _grid(n)
    rng = np.random.default_rng(seed)
    k = np.sqrt(ka2)
    shell = (k >= kmin) & (k <= kmax)
    amp = np.where(shell, np.where(k > 0, k, 1.0) ** amp_slope, 0.0)
    a = amp * np.exp(1j * rng.uniform(0.0, 2.0 * np.pi, size=ka2.shape))
    col = a[0]
    j = np.arange(1, n // 2)
    col[n - j] = np.conj(col[j])
    col[0] = col[0].real
    col[n // 2] = 0.0
    a[0] = col
    return a, ka2


def plan_summary(ctx):
    """The launch shapes the plan autotuner chose for this context."""
    return plan_summary_dict(ctx.plan_report())


def plan_summary_dict(r):
    return {"pass_a": {"radix": r.get("radix_a"), "groups": r["groups_a"], "field_chunks": r["field_chunks_a"]},
            "pass_b": r["chosen"] if r["chosen"] in ("persistent", "split") else f"per_row_pair x{r['groups_b']}",
            "pass_c": r["chosen_c"] if r["chosen_c"] == "persistent"
            else f"per_column_pair x{r['groups_c']}" + (f" ({r['chunks_c']} CTAs per pair)" if r.get("chunks_c", 1) > 1 else "")
            + (f" (teams of {r['team_c']})" if r.get("team_c", 1) > 1 else "")}


def workload_inputs(n):
    """(ps, vz, fp, fz) of the 4096^2 workload (scaled to n for smaller runs)."""
    import numpy as np
    w = WORKLOAD
    s = n / 4096.0
    # energy spectrum E(k) ~ k^-3: |psi| ~ k^-3 (E ~ k^3 |psi|^2), |vz| ~ k^-2
    ps, ka2 = synthetic_field(n, w["ic_kmin"], max(w["ic_kmax"] * s, 4.0), w["ic_slope"], w["ic_seed"])
    vz, _ = synthetic_field(n, w["ic_kmin"], max(w["ic_kmax"] * s, 4.0), w["ic_slope"] + 1.0, w["ic_seed"] + 100)
    ps *= math.sqrt(0.5 / _energy(ps, ka2, 1, n))
    vz *= math.sqrt(0.5 / _energy(vz, ka2, 0, n))
    fkmin, fkmax = max(w["f_kmin"] * s, 2.0), max(w["f_kmax"] * s, 3.0)
    fp, _ = synthetic_field(n, fkmin, fkmax, 0.0, w["f_seed"])
    fz, _ = synthetic_field(n, fkmin, fkmax, 0.0, w["f_seed"] + 100)
    fp *= math.sqrt(1.0 / _energy(fp, ka2, 1, n))
    fz *= math.sqrt(1.0 / _energy(fz, ka2, 0, n))
    return ps, vz, fp, fz, ka2


def make_cparams(n):
    import rot2d3c_gb300 as R
    w = WORKLOAD
    return R.make_params(n=n, nu=w["nu"], hnu=w["hnu"], nn=w["nn"], mm=w["mm"], nuv=w["nu"],
                         hnuv=w["hnu"], nnv=w["nn"], mmv=w["mm"], omega=w["omega"], iflow=0,
                         kup=w["f_kmax"], kdn=w["f_kmin"])


def bench_config(n, world):
    """The `config` of both arms (this one and `--impl reference`): the
    same keys and values, so that the two lines describe one workload."""
    return {"workload": f"single run {n}^2, RK4, dt=1e-4 fixed, nu=1e-5, hnu=0.1 (mm=2), Omega=10, "
                        "IC k^-3 1<=|k|<=100, forcing shell 20-22",
            "n": n, "precision": "FP64 (value: the reference's arithmetic); FP32 path reported in fp32",
            "l2": "working set larger than L2 (state, forcing and six work planes: > 1 GB at 4096^2 FP64)",
            "parallelism": f"replicas x{world}"}


def maybe_spawn(args):
    """--gpus N: under torchrun WORLD_SIZE must equal N; without it, N > 1
    re-launches this script under torch.distributed.run with N ranks."""
    ws = os.environ.get("WORLD_SIZE")
    if ws is not None:
        if int(ws) != args.gpus:
            sys.stderr.write(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={ws}\n")
            sys.exit(2)
        return
    if args.gpus > 1:
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", os.environ.get("MASTER_PORT", "29531"),
               os.path.abspath(__file__)] + sys.argv[1:]
        os.execv(sys.executable, cmd)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"), parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- helpers
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def pass_bytes(n, real_bytes):
    """Algorithmic HBM bytes per launch of passes A, B, C (one substep).
    M = n/3+1 retained kx columns, K = 2(n/3)+1 retained ky rows, c = complex
    element size.  A reads psi, vz on M x K and writes 6 mixed planes M x n;
    B reads the 6 planes and writes 2; C reads 2 planes + c1, c2, ps, vz,
    fp, fz on M x K and writes c1, c2 on M x K."""
    L = n // 3
    M, K = L + 1, 2 * L + 1
    c = 2 * real_bytes
    return {"A": (2 * M * K + 6 * M * n) * c, "B": (6 * M * n + 2 * M * n) * c,
            "C": (2 * M * n + 6 * M * K + 2 * M * K) * c}


def rel_err_fields(a_ps, a_vz, b_ps, b_vz, ka2):
    """Relative L2 errors of omega = k^2 psi and vz (half-plane weighted)."""
    import numpy as np
    two = np.full((a_ps.shape[0], 1), 2.0)
    two[0, 0] = 1.0

    def rl2(x, y):
        return float(np.sqrt(np.sum(two * np.abs(x - y) ** 2) / np.sum(two * np.abs(y) ** 2)))
    return rl2(ka2 * a_ps, ka2 * b_ps), rl2(a_vz, b_vz)


def timed_advance(ctx, steps, dt, torch):
    """Device time of `steps` graph-replayed RK4 steps (CUDA events on the
    context's stream)."""
    import rot2d3c_gb300 as R
    st = torch.cuda.ExternalStream(ctx.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.synchronize()
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches()
    e0.record(st)
    ctx.advance(steps, R.DT_FIXED, dt)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3, ctx.kernel_launches() - l0


def dist_barrier(torch, world):
    if world > 1:
        torch.distributed.barrier()


def dist_max(torch, world, v, device="cuda"):
    """Max over ranks (the slowest replica sets the job's time)."""
    if world <= 1:
        return v
    t = torch.tensor([v], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(torch, world, steps_per_rank, elapsed_s, device="cuda"):
    """Whole-job steps/s of `world` independent replicas: the steps of all
    ranks divided by the slowest rank's time.  Returns (value, max time)."""
    t = dist_max(torch, world, elapsed_s, device)
    return world * steps_per_rank / t, t




def pass_flops(n):
    """Nominal FFT FLOPs per launch of passes A, B, C (5 L log2 L per
    complex transform of length L): A 6 M column IFFTs, B 4 n row
    transforms (per row three packed inverse pairs and one packed forward
    pair), C 2 M column FFTs."""
    M = n // 3 + 1
    per = 5.0 * n * math.log2(n)
    return {"A": 6 * M * per, "B": 4 * n * per, "C": 2 * M * per}


def pass_traffic(n, tag, top):
    """DRAM bytes (read + write) per launch of pass `top` from the committed
    ncu summary profiles/pass_traffic_<tag>_n<n>.json, or None."""
    path = os.path.join(ROOT, "profiles", f"pass_traffic_{tag}_n{n}.json")
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        tr = json.load(f).get(f"k_pass{top}")
    if not tr:
        return None, None
    return tr["dram_read"] + tr["dram_write"], os.path.relpath(path, ROOT) + " (ncu)"


def roofline_of(ms, cnt, n, real_bytes, tag, hbm, peak_kind, peak64=None):
    """HBM roofline of the top pass (algorithmic bytes per launch / CUDA-event
    time per launch) with every pass's figures; for FP64 also the FP64-pipe
    fraction (nominal FFT FLOPs / time against the measured FP64 FMA peak),
    which is what binds that path."""
    pb, pf = pass_bytes(n, real_bytes), pass_flops(n)
    total = sum(ms[j] * cnt[j] for j in range(4))
    passes = {}
    for i, k in enumerate("ABC"):
        d = {"ms_per_launch": ms[i], "algorithmic_bytes": pb[k],
             "achieved_gbs": pb[k] / (ms[i] * 1e-3) / 1e9 if ms[i] > 0 else None,
             "step_share": ms[i] * cnt[i] / total if total > 0 else None}
        d["hbm_frac"] = d["achieved_gbs"] / hbm if d["achieved_gbs"] else None
        if peak64:
            d["fp64_tflops"] = pf[k] / (ms[i] * 1e-3) / 1e12 if ms[i] > 0 else None
            d["fp64_pipe_frac"] = d["fp64_tflops"] / peak64 if d["fp64_tflops"] else None
        passes[k] = d
    top = max("ABC", key=lambda k: passes[k]["ms_per_launch"])
    ach = passes[top]["achieved_gbs"]
    traffic, tsrc = pass_traffic(n, tag, top)
    r = {"bound": "hbm", "kernel": f"k_pass{top} ({'FP64' if real_bytes == 8 else 'FP32'}, n={n})",
         "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_source": peak_kind,
         "traffic": traffic, "traffic_source": tsrc, "algorithmic_bytes_per_launch": pb[top], "passes": passes}
    if peak64:
        r["fp64_pipe"] = {"achieved": passes[top]["fp64_tflops"], "peak": peak64, "unit": "TFLOP/s",
                          "frac": passes[top]["fp64_pipe_frac"],
                          "note": "what binds the FP64 path: nominal FFT FLOPs (5 L log2 L) per launch / "
                                  "launch time, against the FP64 FMA throughput measured on this GPU "
                                  "(r2d3c_fp64_fma_peak)"}
    return r


# ---------------------------------------------------------------- e2e legs
def e2e_roundtrip(ctx, ps, vz, dt, steps, torch, world):
    """The step through the C-ABI with the state owned by the host: every
    step uploads psi-hat and vz-hat from pinned FP64 host buffers
    (r2d3c_set_state), advances one RK4 step (r2d3c_advance) and reads the
    new state back into pinned host buffers (r2d3c_get_state), the way a
    caller that keeps its arrays in host memory would.  The two buffer pairs
    alternate, so each step starts from the previous step's result.  Median
    of three repetitions."""
    import rot2d3c_gb300 as R
    buf = [[torch.empty(a.shape, dtype=torch.complex128).pin_memory().numpy() for a in (ps, vz)]
           for _ in range(2)]
    els = []
    for _ in range(3):
        buf[0][0][...] = ps
        buf[0][1][...] = vz
        ctx.synchronize()
        t0 = time.perf_counter()
        for s in range(steps):
            src, dst = buf[s % 2], buf[(s + 1) % 2]
            ctx.set_state(src[0], src[1])                 # H2D of the state
            ctx.advance(1, R.DT_FIXED, dt)                # one graph-replayed step (dt in, time out)
            R.check(R.load().r2d3c_get_state(ctx._h, R._dptr(dst[0]), R._dptr(dst[1])), "get_state")  # D2H
        els.append(time.perf_counter() - t0)
    el = sorted(els)[1]
    v, el = replica_throughput(torch, world, steps, el)
    S = ps.size * 16
    return {"value": v, "unit": UNIT, "h2d_bytes_per_step": 2 * S + 8, "d2h_bytes_per_step": 2 * S + 16,
            "steps": steps, "repetitions": 3, "statistic": "median",
            "path": "per step: r2d3c_set_state + r2d3c_advance(1) + r2d3c_get_state, pinned host FP64 buffers"}


LOOP = dict(cstep=10, sstep=100, tstep=200, cfl=0.5)


def e2e_main_loop(ctx, ps, vz, steps, torch, world):
    """The drop-in main loop (Rot2D3C.para.f90:393-615) through the C-ABI:
    the state comes from pinned host buffers once, then every step takes its
    dt from the CFL condition (fused into the step), and at a fixed cadence
    (the reference's parameter.inp cadence, cstep 100 / sstep 1000 / tstep
    10000, divided by ten) the host receives cond_check's 30 values, the
    energy spectra and the transfer functions, and the physical psi and vz
    fields; the final state returns to the host."""
    import rot2d3c_gb300 as R
    L = LOOP
    hin = [torch.empty(a.shape, dtype=torch.complex128).pin_memory().numpy() for a in (ps, vz)]
    hout = [torch.empty(a.shape, dtype=torch.complex128).pin_memory().numpy() for a in (ps, vz)]
    hin[0][...] = ps
    hin[1][...] = vz
    n = ctx.n
    calls = {"cond_check": 0, "spectrum+transfers": 0, "fields": 0}
    d2h = 0
    ctx.set_time(0.0)
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.set_state(hin[0], hin[1])
    t = 0.0
    for s in range(steps):
        if s % L["cstep"] == 0:
            ctx.cond_check(t)
            calls["cond_check"] += 1
            d2h += 30 * 8
        if s % L["sstep"] == 0:
            ctx.spectrum()
            ctx.transfers()
            calls["spectrum+transfers"] += 1
            d2h += 5 * (n // 2 + 1) * 8
        if s % L["tstep"] == 0:
            ctx.get_field(R.FIELD_PS)
            ctx.get_field(R.FIELD_VZ)
            calls["fields"] += 1
            d2h += 2 * n * n * 8
        t, _ = ctx.advance(1, R.DT_CFL, L["cfl"])
    R.check(R.load().r2d3c_get_state(ctx._h, R._dptr(hout[0]), R._dptr(hout[1])), "get_state")
    el = time.perf_counter() - t0
    v, el = replica_throughput(torch, world, steps, el)
    S = ps.size * 16
    return {"value": v, "unit": UNIT, "steps": steps, "seconds": el, "calls": calls,
            "h2d_bytes_per_step": 2 * S / steps, "d2h_bytes_per_step": (d2h + 2 * S) / steps,
            "cadence": dict(L, note="reference parameter.inp cadence (cstep 100, sstep 1000, tstep 10000) / 10; "
                                    "dt from the CFL condition every step as in the reference")}


# ---------------------------------------------------------------- ensemble
ENSEMBLE = dict(groups=((512, 64), (1024, 16), (2048, 4)), omega_lo=0.1, omega_hi=100.0, hnu=0.1,
                cfl=0.5, ic_kmin=1.0, ic_kmax=10.0, f_kmin=4.0, f_kmax=6.0, seed=7)


def ensemble_inputs():
    """Per-run (n, params dict, ps, vz, fp, fz) of the batched ensemble:
    Omega log-uniform in [0.1, 100], nu = 1e-3 (256/n)^2, independent IC and
    forcing seeds; IC |u| ~ k^-1 on 1 <= |k| <= 10 with energy 0.5 per field,
    forcing shell 4-6 normalised like iflow = 1."""
    import numpy as np
    e = ENSEMBLE
    rng = np.random.default_rng(e["seed"])
    runs = []
    seed = 1000
    for n, count in e["groups"]:
        for _ in range(count):
            om = float(np.exp(rng.uniform(np.log(e["omega_lo"]), np.log(e["omega_hi"]))))
            nu = 1e-3 * (256.0 / n) ** 2
            ps, ka2 = synthetic_field(n, e["ic_kmin"], e["ic_kmax"], -2.0, seed)
            vz, _ = synthetic_field(n, e["ic_kmin"], e["ic_kmax"], -1.0, seed + 1)
            fp, _ = synthetic_field(n, e["f_kmin"], e["f_kmax"], 0.0, seed + 2)
            fz, _ = synthetic_field(n, e["f_kmin"], e["f_kmax"], 0.0, seed + 3)
            seed += 4
            ps *= math.sqrt(0.5 / _energy(ps, ka2, 1, n))
            vz *= math.sqrt(0.5 / _energy(vz, ka2, 0, n))
            fp *= math.sqrt(1.0 / _energy(fp, ka2, 1, n))
            fz *= math.sqrt(1.0 / _energy(fz, ka2, 0, n))
            prm = dict(n=n, nu=nu, nuv=nu, hnu=e["hnu"], hnuv=e["hnu"], nn=1, mm=2, nnv=1, mmv=2, omega=om,
                       iflow=0, cfl=e["cfl"], kup=e["f_kmax"], kdn=e["f_kmin"])
            runs.append((n, prm, ps, vz, fp, fz))
    return runs


def budget_residuals(S):
    """Energy-budget residual of every run from cond_check samples S
    [sample][run][30] (BalanceTest_Rot2D3C.py: d/dt (E + Ez)/2 = inj - diss):
    |mean(dE/dt - (inj - diss))| / mean|inj| over the interior samples, dE/dt
    by centred differences of the samples."""
    import numpy as np
    tm = S[:, :, 0]
    etot = 0.5 * (S[:, :, 1] + S[:, :, 2])
    inj = S[:, :, 3] + S[:, :, 4]
    diss = S[:, :, 5] + S[:, :, 6] + S[:, :, 7] + S[:, :, 8]
    out = []
    for i in range(S.shape[1]):
        dE = np.gradient(etot[:, i], tm[:, i])
        r = dE - (inj[:, i] - diss[:, i])
        out.append(float(np.abs(np.mean(r[1:-1])) / max(np.mean(np.abs(inj[:, i])), 1e-300)))
    return np.array(out)


def run_ensemble(args, torch, rank=0, world=1):
    """runs/s of the batched ensemble (every run advances `steps` CFL steps,
    one CUDA graph per step holding every size group) and each run's
    energy-budget residual.  With several ranks the runs are partitioned by
    cost (rot2d3c_gb300.partition) and the per-run residuals are gathered
    on the host; the time is the slowest rank's."""
    import numpy as np
    import rot2d3c_gb300 as R
    from rot2d3c_gb300 import partition as P
    runs = ensemble_inputs()
    mine = P.partition([r[0] for r in runs], world)[rank]
    groups = []
    for n, _ in ENSEMBLE["groups"]:
        ids = [i for i in mine if runs[i][0] == n]
        if ids:
            groups.append((n, [R.make_params(**runs[i][1]) for i in ids]))
    order = [i for n, _ in ENSEMBLE["groups"] for i in mine if runs[i][0] == n]  # ensemble run -> global run
    ens = R.Ensemble(groups, R.FP32)
    for j, i in enumerate(order):
        n, prm, ps, vz, fp, fz = runs[i]
        ens.set_state(j, ps, vz)
        ens.set_forcing(j, fp, fz)
        ens.set_time(j, 0.0)
    # budget: cond_check after every step over 100 steps (outside the timed
    # region); the residual from every sample and from every tenth sample
    # (cstep 10) separates the finite-difference error of dE/dt from the
    # budget's own mismatch
    samples = []
    t = np.zeros(len(order))
    for k in range(101):
        samples.append(np.array([ens.cond_check(j, t[j]) for j in range(len(order))]))
        if k < 100:
            t = ens.advance(1, R.DT_CFL, ENSEMBLE["cfl"])
    S = np.array(samples)
    r1, r10 = budget_residuals(S), budget_residuals(S[::10])
    res_local = {i: (float(a), float(b)) for i, a, b in zip(order, r1, r10)}
    both = np.array(P.gather_by_run(res_local, world, len(runs)))
    resid, resid10 = both[:, 0], both[:, 1]
    # timed: `steps` more steps of every run
    K = args.ensemble_steps
    ens.advance(3, R.DT_CFL, ENSEMBLE["cfl"])  # warm-up
    l0 = ens.kernel_launches()
    dist_barrier(torch, world)
    torch.cuda.synchronize()
    t0 = time_mod.perf_counter()
    ens.advance(K, R.DT_CFL, ENSEMBLE["cfl"])
    el = dist_max(torch, world, time_mod.perf_counter() - t0)
    worst = int(np.argmax(resid))
    worst10 = int(np.argmax(resid10))
    out = {"value": len(runs) / el, "unit": f"runs/s ({K} RK4 steps per run)",
           "runs": len(runs), "groups": [list(g) for g in ENSEMBLE["groups"]], "steps_per_run": K,
           "seconds": el, "gpu_launches": ens.kernel_launches() - l0, "dtype": "f32 (FP64 reductions)",
           "ranks": world, "partition": "runs dealt by cost n^2 log2 n (LPT), diagnostics gathered on the host",
           "plan": {str(g["n"]): dict(plan_summary_dict(g["plan"]), policy=g["plan"].get("policy"))
                    for g in ens.plan_report()},
           "budget_residual": {"median": float(np.median(resid)), "max": float(resid.max()),
                               "worst_run": {"index": worst, "n": runs[worst][0],
                                             "omega": runs[worst][1]["omega"]},
                               "cstep10": {"median": float(np.median(resid10)), "max": float(resid10.max()),
                                           "worst_run": {"index": worst10, "n": runs[worst10][0],
                                                         "omega": runs[worst10][1]["omega"]}},
                               "definition": "|mean(dE_tot/dt - (inj - diss))| / mean|inj| over 100 steps, "
                                             "dE/dt by centred differences of cond_check samples taken every "
                                             "step (cstep10: every 10 steps)"},
           "config": "64 x 512^2 + 16 x 1024^2 + 4 x 2048^2, Omega log-uniform [0.1,100], nu=1e-3(256/n)^2, "
                     "hnu=0.1, CFL=0.5, forcing shell 4-6, independent seeds"}
    ens.destroy()
    return out


# ---------------------------------------------------------------- precision study
CONFIG4 = dict(n=8192, steps=50, nu=2e-6, hnu=0.1, omega=1.0, ic_kmin=1.0, ic_kmax=200.0, f_kmin=30.0,
               f_kmax=32.0, cfl=0.5, seed=81)


def run_precision_study(args, torch):
    """The 8192^2 precision study: 50 CFL-controlled RK4 steps of the FP64
    and the FP32 path from the same seeded state (k^-3 initial spectrum on
    1 <= |k| <= 200, forcing shell 30-32, nu = 2e-6, hnu = 0.1, Omega = 1):
    steps/s and per-pass times of both, the FP32 path's relative L2 error
    of omega and vz against FP64, and its per-shell energy-spectrum error."""
    import numpy as np
    import rot2d3c_gb300 as R
    c4 = CONFIG4
    n = c4["n"]
    ps, ka2 = synthetic_field(n, c4["ic_kmin"], c4["ic_kmax"], -3.0, c4["seed"])
    vz, _ = synthetic_field(n, c4["ic_kmin"], c4["ic_kmax"], -2.0, c4["seed"] + 100)
    fp, _ = synthetic_field(n, c4["f_kmin"], c4["f_kmax"], 0.0, c4["seed"] + 1)
    fz, _ = synthetic_field(n, c4["f_kmin"], c4["f_kmax"], 0.0, c4["seed"] + 101)
    ps *= math.sqrt(0.5 / _energy(ps, ka2, 1, n))
    vz *= math.sqrt(0.5 / _energy(vz, ka2, 0, n))
    fp *= math.sqrt(1.0 / _energy(fp, ka2, 1, n))
    fz *= math.sqrt(1.0 / _energy(fz, ka2, 0, n))
    cp = R.make_params(n=n, nu=c4["nu"], hnu=c4["hnu"], nn=1, mm=2, nuv=c4["nu"], hnuv=c4["hnu"], nnv=1, mmv=2,
                       omega=c4["omega"], iflow=0, kup=c4["f_kmax"], kdn=c4["f_kmin"])
    out = {}
    for prec, tag in ((R.FP64, "fp64"), (R.FP32, "fp32")):
        c = R.Context(cp, prec)
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        st = torch.cuda.ExternalStream(c.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c.synchronize()
        l0 = c.kernel_launches()
        e0.record(st)
        t, dt = c.advance(c4["steps"], R.DT_CFL, c4["cfl"])
        e1.record(st)
        e1.synchronize()
        el = e0.elapsed_time(e1) / 1e3
        launches = c.kernel_launches() - l0
        state = c.get_state()
        ek = c.spectrum()[0]
        ms, cnt = c.profile_passes(2, dt)
        out[tag] = {"value": c4["steps"] / el, "unit": UNIT, "ms_per_step": 1e3 * el / c4["steps"],
                    "gpu_launches": launches, "time": t, "last_dt": dt,
                    "passes_ms_per_launch": dict(zip("ABC", ms[:3])), "state": state, "ek": ek}
        c.destroy()
    a64, b64 = out["fp64"].pop("state")
    a32, b32 = out["fp32"].pop("state")
    ek64, ek32 = out["fp64"].pop("ek"), out["fp32"].pop("ek")
    ew, ev = rel_err_fields(a32, b32, a64, b64, ka2)
    live = ek64 > 1e-14 * ek64.max()
    rel = np.abs(ek32[live] - ek64[live]) / ek64[live]
    return {"config": f"{n}^2, RK4, {c4['steps']} CFL steps (cfl {c4['cfl']}), nu={c4['nu']}, hnu={c4['hnu']} (mm=2), "
                      f"Omega={c4['omega']}, IC k^-3 1<=|k|<=200, forcing shell 30-32",
            "fp64": out["fp64"], "fp32": out["fp32"], "fp32_speedup": out["fp32"]["value"] / out["fp64"]["value"],
            "err_fp32_vs_fp64": {"rel_l2_omega": ew, "rel_l2_vz": ev,
                                 "spectrum_shell_rel": {"max": float(rel.max()), "median": float(np.median(rel)),
                                                        "shells": int(live.sum())}}}


# ---------------------------------------------------------------- closure
# the network is evaluated before every second LES step (its tendencies held
# for two steps): on this configuration as close to the filtered DNS as every
# step, at 1.25 times the gain (every fourth step: worse energy-weighted error)
CLOSURE = dict(nf=2048, nc=256, omega=1.0, nu=2e-5, hnu=1.0, nsnap=1000, snap_every=20, spinup=10000,
               train_steps=6000, batch=32, lr=5e-4, les_steps=4000, cfl=0.5, seed=1, every=2)


CLOSURE_SMALL = dict(CLOSURE, nf=512, nc=128, nu=2e-4, nsnap=64, snap_every=5, spinup=200, train_steps=40,
                     les_steps=200, spec_every=20, every=1)

# The full-size closure experiment (2048^2 DNS -> 256^2 LES, nu = 5e-6, 2000
# snapshots, 20k Adam steps of batch 32 at lr 1e-3, 5000 LES steps), once per
# Omega in {1, 10}; the
# reference's default hypoviscosity (parameter.inp: hnu = 1, mm = 2) keeps
# the forced flow statistically steady.  Several minutes: --closure-full.
CLOSURE_FULL = dict(nf=2048, nc=256, nu=5e-6, hnu=1.0, nsnap=2000, snap_every=20, spinup=10000,
                    train_steps=20000, batch=32, lr=1e-3, les_steps=5000, cfl=0.5, seed=1)


def run_closure_full():
    """The full-size closure experiment for Omega = 1 and Omega = 10."""
    return {f"omega_{om:g}": run_closure(cfg=dict(CLOSURE_FULL, omega=om)) for om in (1.0, 10.0)}


def run_closure(small=False, cfg=None):
    """The learned-closure experiment (rot2d3c_gb300.les): FP32 DNS at 2048^2,
    filtered snapshots, CNN training, then the 256^2 LES with the network in
    the loop against the plain and hyperviscous coarse solvers and the
    filtered DNS over the same physical time.  The gain is the DNS's GPU
    seconds over the LES's for that time."""
    from rot2d3c_gb300.les import run_experiment, step_timing
    cfg = cfg or (CLOSURE_SMALL if small else CLOSURE)
    r = run_experiment(**cfg)
    tr = r["training"]
    nshow = 16
    # GPU time per coarse step of each LES schedule (graph replay, CUDA events)
    steps_us = step_timing(nc=cfg["nc"], steps=200, nu=cfg["nu"], hnu=cfg["hnu"], omega=cfg["omega"],
                           cfl=cfg["cfl"])
    return {"les_vs_dns_gain": r["les"]["gain"], "unit": "DNS GPU-s / LES GPU-s (same physical time)",
            "step_us": dict({k: round(v, 2) for k, v in steps_us.items()},
                            note="us per coarse step: plain solver; network before every step, every second "
                                 "step, one step behind beside the step (overlap)"),
            "dns": r["dns"], "les": r["les"], "spectrum_error": r["spectrum_error"],
            "spectrum_error_per_start": r["spectrum_error_per_start"], "skill": r["skill"],
            "spectra_shells_0_15": {k: [float(f"{x:.4g}") for x in v[:nshow]] for k, v in r["spectra"].items()},
            "training": dict(tr, ms_per_step=1e3 * tr["train_s"] / tr["steps"],
                             samples_per_s=tr["steps"] * tr["batch"] / tr["train_s"]),
            "config": dict(cfg, network="6 x conv3x3 8-32-32-32-32-32-2, GELU, BF16 tensor-core MMA, FP32 master "
                                           "weights, Adam; dataset and LES on GPU"),
            "total_s": r["total_s"]}


# ---------------------------------------------------------------- CPU legs
CPU_FFT_NOTE = ("the C/OpenMP restatement's own radix-2 FFT (not FFTW, which the reference links: FFTW would "
                "be faster by an unmeasured factor)")


def oracle_params(n):
    from oracle import rot2d3c_oracle as O
    w = WORKLOAD
    return O.Params(n=n, nu=w["nu"], hnu=w["hnu"], nn=w["nn"], mm=w["mm"], nuv=w["nu"], hnuv=w["hnu"],
                    nnv=w["nn"], mmv=w["mm"], omega=w["omega"], iflow=0)


def cpu_leg(n, ps, vz, fp, fz, steps, budget_s=30.0):
    """The C/OpenMP restatement of the reference step (oracle/cpu) from the
    workload's initial state for `steps` steps on all host cores: the state
    after `steps` steps (to check both GPU paths against) and, timed inside
    that run, a bounded sample of its steps (the CPU baseline); plus one step
    on one thread."""
    from oracle import cpu_oracle as CO
    p = oracle_params(n)
    dt = WORKLOAD["dt"]
    th = CO.max_threads()
    a, b, _ = CO.run(p, ps, vz, fp, fz, 1, dt, False, th)      # untimed first step
    t0 = time.perf_counter()
    a, b, _ = CO.run(p, a, b, fp, fz, 1, dt, False, th)
    per = time.perf_counter() - t0
    k = max(1, min(steps - 2, int(budget_s / max(per, 1e-6)) - 1)) if steps > 2 else 0
    dtk = 0.0
    if k:
        t0 = time.perf_counter()
        a, b, _ = CO.run(p, a, b, fp, fz, k, dt, False, th)
        dtk = time.perf_counter() - t0
    rest = steps - 2 - k
    if rest > 0:
        a, b, _ = CO.run(p, a, b, fp, fz, rest, dt, False, th)
    t0 = time.perf_counter()
    CO.run(p, a, b, fp, fz, 1, dt, False, 1)
    dt1 = time.perf_counter() - t0
    v = (k + 1) / (dtk + per)
    cpu = {"value": v, "unit": UNIT, "cores": th, "kind": "port", "value_1thread": 1.0 / dt1,
           "sample": f"steps 2..{k + 2} of a {steps}-step run at {n}^2 FP64 from the workload's initial state, "
                     f"{th} threads (MPI ranks: 1, threads instead of MPI); C/OpenMP restatement of the reference "
                     f"step with the reference's cost structure (32 C2R + 8 R2C 2-D transforms per fixed-dt step), "
                     f"FFT: {CPU_FFT_NOTE}; value_1thread: 1 step on 1 thread"}
    return cpu, (a, b)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    n = args.n
    ps, vz, fp, fz, _ = workload_inputs(n)
    from oracle import cpu_oracle as CO
    p = oracle_params(n)
    w = WORKLOAD
    th = CO.max_threads()
    warm = max(0, min(args.warmup, 5))  # the requested warm-up steps, at most 5 (about 3 s on 16 cores)
    a, b = ps, vz
    if warm:
        a, b, _ = CO.run(p, a, b, fp, fz, warm, w["dt"], False, th)
    # bounded sample: at most args.steps steps or ~60 s of CPU work
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        a, b, _ = CO.run(p, a, b, fp, fz, 1, w["dt"], False, th)
        done += 1
        if time.perf_counter() - t0 > 60.0:
            break
    el = time.perf_counter() - t0
    v = done / el
    sample = (f"{done} of {args.steps} requested RK4 steps at {n}^2 FP64 (bounded to ~60 s) after {warm} "
              f"warm-up steps, C/OpenMP restatement of the reference step, {th} threads, MPI ranks: 1; "
              f"FFT: {CPU_FFT_NOTE}")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": done, "warmup": warm, "ms_per_step": 1e3 * el / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(n, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": th, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- main arm
def main():
    args = parse()
    maybe_spawn(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args)
        return
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np  # noqa: F401
    import torch
    if world > 1:
        torch.cuda.set_device(0)
        torch.distributed.init_process_group("nccl")
    import rot2d3c_gb300 as R
    from rot2d3c_gb300 import build as B
    B.build()
    R.load()

    n = args.n
    dt = WORKLOAD["dt"]
    K, W = args.steps, max(3, args.warmup)
    ps, vz, fp, fz, ka2 = workload_inputs(n)
    cp = make_cparams(n)
    hbm, peak_kind = measured_peaks()

    def make(prec):
        c = R.Context(cp, prec)
        c.set_state(ps, vz)
        c.set_forcing(fp, fz)
        c.set_time(0.0)
        return c

    # ---- accuracy runs (untimed): both paths from the same state, err_steps steps
    c64 = None if args.no_fp64 else make(R.FP64)
    c32 = None if (args.no_fp32 and not args.no_fp64) else make(R.FP32)
    s64 = s32 = None
    if c64 is not None:
        c64.advance(args.err_steps, R.DT_FIXED, dt)
        s64 = c64.get_state()
    if c32 is not None:
        c32.advance(args.err_steps, R.DT_FIXED, dt)
        s32 = c32.get_state()

    # ---- FP64 drop-in path: the headline
    v64 = el64 = launches64 = roofline = e2e = e2e_loop = plan64 = clocks = None
    if c64 is not None:
        c64.advance(W, R.DT_FIXED, dt)
        dist_barrier(torch, world)
        with ClockSampler(local if world == 1 else 0) as clk:
            el64, launches64 = timed_advance(c64, K, dt, torch)
            dist_barrier(torch, world)
        v64, el64 = replica_throughput(torch, world, K, el64)
        clocks = clk.summary()
        ms64, cnt64 = c64.profile_passes(min(K, 4), dt)
        peak64 = R.fp64_fma_peak()
        roofline = roofline_of(ms64, cnt64, n, 8, "fp64", hbm, peak_kind, peak64)
        e2e = e2e_roundtrip(c64, ps, vz, dt, min(K, args.e2e_steps), torch, world)
        e2e_loop = e2e_main_loop(c64, ps, vz, args.loop_steps, torch, world) if args.loop_steps > 0 else None
        plan64 = plan_summary(c64)
        c64.destroy()

    # ---- FP32 path
    fp32 = None
    if c32 is not None:
        K32 = args.fp32_steps or K
        c32.advance(W, R.DT_FIXED, dt)
        dist_barrier(torch, world)
        with ClockSampler(local if world == 1 else 0) as clk32:
            el32, launches32 = timed_advance(c32, K32, dt, torch)
            dist_barrier(torch, world)
        v32, el32 = replica_throughput(torch, world, K32, el32)
        ms32, cnt32 = c32.profile_passes(min(K32, 20), dt)
        fp32 = {"value": v32, "unit": UNIT, "ms_per_step": 1e3 * el32 / K32, "steps": K32,
                "dtype": "f32 (compensated twiddles, FP64 reductions)",
                "fp32_speedup": v32 / v64 if v64 else None, "gpu_launches": launches32,
                "roofline": roofline_of(ms32, cnt32, n, 4, "fp32", hbm, peak_kind),
                "e2e": e2e_roundtrip(c32, ps, vz, dt, min(K32, 50), torch, world),
                "clocks": clk32.summary(), "plan": plan_summary(c32)}
        if s64 is not None:
            ew, ev = rel_err_fields(s32[0], s32[1], s64[0], s64[1], ka2)
            fp32["err_vs_fp64"] = {"rel_l2_omega": ew, "rel_l2_vz": ev, "after_steps": args.err_steps}
        c32.destroy()
    if c64 is None:  # FP32-only profiling run: the line reports the FP32 leg
        v64, el64, K, launches64 = fp32["value"], fp32["ms_per_step"] * K32 / 1e3, K32, fp32["gpu_launches"]
        roofline, e2e, clocks, plan64 = fp32["roofline"], fp32["e2e"], fp32["clocks"], fp32["plan"]

    ensemble = None if args.no_ensemble else run_ensemble(args, torch, rank, world)
    precision = None
    if rank == 0 and world == 1 and not args.no_precision_study:
        precision = run_precision_study(args, torch)

    cpu = None
    err_oracle = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.oracle_steps > 0:
        cpu, (oa, ob) = cpu_leg(n, ps, vz, fp, fz, args.oracle_steps)
        if args.oracle_steps == args.err_steps:
            err_oracle = {"after_steps": args.err_steps, "oracle": "C/OpenMP restatement (oracle/cpu), FP64"}
            if s64 is not None:
                ew, ev = rel_err_fields(s64[0], s64[1], oa, ob, ka2)
                err_oracle["fp64"] = {"rel_l2_omega": ew, "rel_l2_vz": ev}
            if s32 is not None:
                ew, ev = rel_err_fields(s32[0], s32[1], oa, ob, ka2)
                err_oracle["fp32"] = {"rel_l2_omega": ew, "rel_l2_vz": ev}
                fp32["err_vs_oracle"] = err_oracle["fp32"]
    closure = closure_full = None
    if rank == 0 and world == 1 and not args.no_closure:
        closure = run_closure(args.closure_small)
    if rank == 0 and world == 1 and args.closure_full:
        closure_full = run_closure_full()

    line = {"metric": METRIC, "value": v64, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * el64 / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if not args.no_fp64 else "f32 (FP64 leg skipped)",
            "data": "synthetic", "config": bench_config(n, world), "plan": plan64,
            "gpu_launches": launches64, "roofline": roofline, "clocks": clocks, "e2e": e2e,
            "e2e_loop": e2e_loop, "err_vs_oracle": err_oracle, "fp32": fp32, "precision_8192": precision,
            "ensemble": ensemble, "closure": closure, "closure_full": closure_full, "cpu_baseline": cpu}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
