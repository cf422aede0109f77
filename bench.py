#!/usr/bin/env python
"""Benchmark of the Rot2D3C RK4 time step on GB300.

Workload: a single large run at n = 4096^2, RK order 4, fixed dt = 1e-4,
nu = nuv = 1e-5 (nn = 1), hypoviscosity hnu = hnuv = 0.1 (nabla^-4, mm = 2),
Omega = 10, a seeded random-phase initial spectrum ~ k^-3 for 1 <= |k| <= 100
(energy(ps,1) = energy(vz,0) = 0.5) and a seeded, time-constant random-phase
forcing in the shell 20 <= |k| <= 22 normalised like iflow = 1
(energy(fp,1) = energy(fz,0) = 1).  All inputs are synthetic.

One bench step = one RK4 step.  The headline `value` is the FP32 path
(FP32 fields and transforms with compensated twiddles, FP64 reductions); the
FP64 drop-in path is measured on the same workload and reported in `fp64`,
with the relative L2 error of omega and vz of the FP32 path against FP64
after 100 steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: one field does not shard (replicas only); under torchrun every
rank runs its own replica and `value` counts the steps of all ranks.
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
    ap.add_argument("--fp64-steps", type=int, default=0, help="timed FP64 steps (default: --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--err-steps", type=int, default=100)
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--ensemble-steps", type=int, default=500)
    ap.add_argument("--no-closure", action="store_true")
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
    return {"pass_a": {"groups": r["groups_a"], "field_chunks": r["field_chunks_a"]},
            "pass_b": r["chosen"] if r["chosen"] == "persistent" else f"per_row_pair x{r['groups_b']}",
            "pass_c": r["chosen_c"] if r["chosen_c"] == "persistent" else f"per_column_pair x{r['groups_c']}"}


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


def fft_flops_per_step(n):
    """Nominal FFT FLOPs of one RK4 step of the fused path (5 L log2 L per
    complex transform of length L): per substep 6 M column IFFTs (A), 4 n
    packed row transforms (B), 2 M column FFTs (C)."""
    M = n // 3 + 1
    per = 5.0 * n * math.log2(n)
    return 4 * (6 * M + 4 * n + 2 * M) * per


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


def run_ensemble(args, torch):
    """runs/s of the batched ensemble (all runs advance `steps` CFL steps in
    one CUDA graph per step) and each run's total-energy budget residual
    (BalanceTest_Rot2D3C.py: d/dt (E + Ez)/2 = inj - diss) over 100 steps."""
    import numpy as np
    import rot2d3c_gb300 as R
    runs = ensemble_inputs()
    groups = []
    for n, count in ENSEMBLE["groups"]:
        groups.append((n, [R.make_params(**r[1]) for r in runs if r[0] == n]))
    ens = R.Ensemble(groups, R.FP32)
    for i, (n, prm, ps, vz, fp, fz) in enumerate(runs):
        ens.set_state(i, ps, vz)
        ens.set_forcing(i, fp, fz)
        ens.set_time(i, 0.0)
    # budget: cond_check every 10 steps over 100 steps (outside the timed region)
    samples = []
    t = np.zeros(len(runs))
    for k in range(11):
        samples.append(np.array([ens.cond_check(i, t[i]) for i in range(len(runs))]))
        if k < 10:
            t = ens.advance(10, R.DT_CFL, ENSEMBLE["cfl"])
    S = np.array(samples)  # [sample][run][30]
    time = S[:, :, 0]
    etot = 0.5 * (S[:, :, 1] + S[:, :, 2])
    inj = S[:, :, 3] + S[:, :, 4]
    diss = S[:, :, 5] + S[:, :, 6] + S[:, :, 7] + S[:, :, 8]
    resid = []
    for i in range(len(runs)):
        dE = np.gradient(etot[:, i], time[:, i])
        r = dE - (inj[:, i] - diss[:, i])
        resid.append(float(np.abs(np.mean(r[1:-1])) / max(np.mean(np.abs(inj[:, i])), 1e-300)))
    resid = np.array(resid)
    # timed: `steps` more steps of every run
    K = args.ensemble_steps
    ens.advance(3, R.DT_CFL, ENSEMBLE["cfl"])  # warm-up
    l0 = ens.kernel_launches()
    torch.cuda.synchronize()
    t0 = time_mod.perf_counter()
    ens.advance(K, R.DT_CFL, ENSEMBLE["cfl"])
    el = time_mod.perf_counter() - t0
    out = {"value": len(runs) / el, "unit": f"runs/s ({K} RK4 steps per run)",
           "runs": len(runs), "groups": [list(g) for g in ENSEMBLE["groups"]], "steps_per_run": K,
           "seconds": el, "gpu_launches": ens.kernel_launches() - l0, "dtype": "f32 (FP64 reductions)",
           "plan": {str(g["n"]): plan_summary_dict(g["plan"]) for g in ens.plan_report()},
           "budget_residual": {"median": float(np.median(resid)), "max": float(resid.max()),
                               "definition": "|mean(dE_tot/dt - (inj - diss))| / mean|inj| over 100 steps, "
                                             "cond_check every 10 steps"},
           "config": "64 x 512^2 + 16 x 1024^2 + 4 x 2048^2, Omega log-uniform [0.1,100], nu=1e-3(256/n)^2, "
                     "hnu=0.1, CFL=0.5, forcing shell 4-6, independent seeds"}
    ens.destroy()
    return out


# ---------------------------------------------------------------- closure
CLOSURE = dict(nf=2048, nc=256, omega=1.0, nu=2e-5, hnu=1.0, nsnap=1000, snap_every=20, spinup=10000,
               train_steps=6000, batch=32, lr=5e-4, les_steps=4000, cfl=0.5, seed=1)


CLOSURE_SMALL = dict(CLOSURE, nf=512, nc=128, nu=2e-4, nsnap=64, snap_every=5, spinup=200, train_steps=40,
                     les_steps=200, spec_every=20)


def run_closure(small=False):
    """The learned-closure experiment (rot2d3c_gb300.les): FP32 DNS at 2048^2,
    filtered snapshots, CNN training, then the 256^2 LES with the network in
    the loop against the plain and hyperviscous coarse solvers and the
    filtered DNS over the same physical time.  The gain is the DNS's GPU
    seconds over the LES's for that time."""
    from rot2d3c_gb300.les import run_experiment
    cfg = CLOSURE_SMALL if small else CLOSURE
    r = run_experiment(**cfg)
    tr = r["training"]
    return {"les_vs_dns_gain": r["les"]["gain"], "unit": "DNS GPU-s / LES GPU-s (same physical time)",
            "dns": r["dns"], "les": r["les"], "spectrum_error": r["spectrum_error"],
            "training": dict(tr, ms_per_step=1e3 * tr["train_s"] / tr["steps"],
                             samples_per_s=tr["steps"] * tr["batch"] / tr["train_s"]),
            "config": dict(cfg, network="6 x conv3x3 8-32-32-32-32-32-2, GELU, BF16 tensor-core MMA, FP32 master "
                                           "weights, Adam; dataset and LES on GPU"),
            "total_s": r["total_s"]}


# ---------------------------------------------------------------- CPU legs
def cpu_baseline(n, ps, vz, fp, fz, budget_s=20.0):
    """The C/OpenMP restatement of the reference step (oracle/cpu) on all host
    cores: a bounded sample of the same workload."""
    from oracle import cpu_oracle as CO
    from oracle import rot2d3c_oracle as O
    w = WORKLOAD
    p = O.Params(n=n, nu=w["nu"], hnu=w["hnu"], nn=w["nn"], mm=w["mm"], nuv=w["nu"], hnuv=w["hnu"],
                 nnv=w["nn"], mmv=w["mm"], omega=w["omega"], iflow=0)
    th = CO.max_threads()
    t0 = time.perf_counter()
    a, b, _ = CO.run(p, ps, vz, fp, fz, 1, w["dt"], False, th)
    t1 = time.perf_counter()
    per = t1 - t0
    k = max(1, min(20, int(budget_s / max(per, 1e-6)) - 1))
    t0 = time.perf_counter()
    CO.run(p, a, b, fp, fz, k, w["dt"], False, th)
    dt = time.perf_counter() - t0
    # one thread, one step (the reference's per-rank work without MPI)
    t0 = time.perf_counter()
    CO.run(p, a, b, fp, fz, 1, w["dt"], False, 1)
    dt1 = time.perf_counter() - t0
    return {"value": k / dt, "unit": UNIT, "cores": th, "kind": "port", "value_1thread": 1.0 / dt1,
            "sample": f"{k} RK4 steps at {n}^2 FP64 (after 1 untimed), C/OpenMP restatement of the "
                      f"reference step (35 C2R + 8 R2C per step as in the reference), {th} threads; "
                      "value_1thread: 1 step on 1 thread; MPI ranks: 1 (threads instead of MPI)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    n = args.n
    ps, vz, fp, fz, _ = workload_inputs(n)
    from oracle import cpu_oracle as CO
    from oracle import rot2d3c_oracle as O
    w = WORKLOAD
    p = O.Params(n=n, nu=w["nu"], hnu=w["hnu"], nn=w["nn"], mm=w["mm"], nuv=w["nu"], hnuv=w["hnu"],
                 nnv=w["nn"], mmv=w["mm"], omega=w["omega"], iflow=0)
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
              f"warm-up steps, "
              f"C/OpenMP restatement of the reference step, {th} threads, MPI ranks: 1")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": done, "warmup": warm, "ms_per_step": 1e3 * el / done, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"single run {n}^2, RK4, dt=1e-4 fixed, nu=1e-5, hnu=0.1, Omega=10, "
                                   "IC k^-3 1<=|k|<=100, forcing shell 20-22", "n": n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": th, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- main arm
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args)
        return
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
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

    # ---- FP32 path: accuracy run, then timing
    c32 = R.Context(cp, R.FP32)
    c32.set_state(ps, vz)
    c32.set_forcing(fp, fz)
    out = {}
    if not args.no_fp64:
        c64 = R.Context(cp, R.FP64)
        c64.set_state(ps, vz)
        c64.set_forcing(fp, fz)
        c64.advance(args.err_steps, R.DT_FIXED, dt)
        c32.advance(args.err_steps, R.DT_FIXED, dt)
        a64, b64 = c64.get_state()
        a32, b32 = c32.get_state()
        ew, ev = rel_err_fields(a32, b32, a64, b64, ka2)
        out["err"] = {"rel_l2_omega": ew, "rel_l2_vz": ev, "after_steps": args.err_steps}
        del a64, b64, a32, b32

    c32.advance(W, R.DT_FIXED, dt)
    dist_barrier(torch, world)
    with ClockSampler(local if world == 1 else 0) as clk:
        el32, launches32 = timed_advance(c32, K, dt, torch)
        dist_barrier(torch, world)
    v32, el32 = replica_throughput(torch, world, K, el32)
    clocks = clk.summary()

    # per-pass device times (CUDA events around each launch, separate pass)
    ms32, cnt32 = c32.profile_passes(min(K, 20), dt)
    hbm, peak_kind = measured_peaks()
    pb = pass_bytes(n, 4)
    passes = {k: {"ms_per_launch": ms32[i], "algorithmic_bytes": pb[k],
                  "achieved_gbs": pb[k] / (ms32[i] * 1e-3) / 1e9 if ms32[i] > 0 else None}
              for i, k in enumerate("ABC")}
    top = max("ABC", key=lambda k: passes[k]["ms_per_launch"])
    ach = passes[top]["achieved_gbs"]
    traffic = None
    tpath = os.path.join(ROOT, "profiles", f"pass_traffic_fp32_n{n}.json")
    if os.path.exists(tpath):  # DRAM bytes per launch from the committed ncu capture
        with open(tpath) as f:
            tr = json.load(f).get(f"k_pass{top}")
        if tr:
            traffic = tr["dram_read"] + tr["dram_write"]
    roofline = {"bound": "hbm", "kernel": f"k_pass{top} (FP32, n={n})", "achieved": ach, "peak": hbm,
                "unit": "GB/s", "frac": ach / hbm, "peak_source": peak_kind,
                "traffic": traffic, "traffic_source": "profiles/pass_traffic_fp32_n4096.json (ncu)",
                "algorithmic_bytes_per_launch": pass_bytes(n, 4)[top], "passes": passes,
                "step_share": {k: ms32[i] * cnt32[i] / sum(ms32[j] * cnt32[j] for j in range(4))
                               for i, k in enumerate("ABC")}}

    # ---- e2e through the C-ABI with host buffers (FP32 path): the state goes
    # in from and comes back to pinned host FP64 buffers (allocated before the
    # timed region, as a caller that reuses its buffers would), and every step
    # is one r2d3c_advance call (coefficients and dt in, time and dt out)
    e2e_steps = min(K, 50)
    hp_in = [torch.empty(a.shape, dtype=torch.complex128).pin_memory().numpy() for a in (ps, vz)]
    hp_out = [torch.empty(a.shape, dtype=torch.complex128).pin_memory().numpy() for a in (ps, vz)]
    hp_in[0][...] = ps
    hp_in[1][...] = vz
    # three repetitions, the median counts (host-side jitter of single runs)
    els = []
    for _ in range(3):
        c32.synchronize()
        t0 = time.perf_counter()
        c32.set_state(hp_in[0], hp_in[1])           # H2D of the state
        for _ in range(e2e_steps):
            c32.advance(1, R.DT_FIXED, dt)          # H2D coefficients and dt, launch, D2H time and dt
        R.check(R.load().r2d3c_get_state(c32._h, R._dptr(hp_out[0]), R._dptr(hp_out[1])), "get_state")  # D2H
        els.append(time.perf_counter() - t0)
    el_e2e = sorted(els)[1]
    ve2e, el_e2e = replica_throughput(torch, world, e2e_steps, el_e2e)
    S = (n // 2 + 1) * n * 16
    e2e = {"value": ve2e, "unit": UNIT,
           "h2d_bytes_per_step": (2 * S + 8 * e2e_steps) / e2e_steps,
           "d2h_bytes_per_step": (2 * S + 16 * e2e_steps) / e2e_steps,
           "steps": e2e_steps, "repetitions": 3, "statistic": "median",
           "path": "r2d3c_set_state + per-step r2d3c_advance(1) + r2d3c_get_state (pinned host FP64 buffers)"}

    # ---- FP64 drop-in path
    fp64 = None
    if not args.no_fp64:
        K64 = args.fp64_steps or K
        c64.advance(W, R.DT_FIXED, dt)
        el64, l64 = timed_advance(c64, K64, dt, torch)
        v64, el64 = replica_throughput(torch, world, K64, el64)
        ms64, cnt64 = c64.profile_passes(min(K64, 4), dt)
        peak64 = R.fp64_fma_peak()
        flops = fft_flops_per_step(n)
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": 1e3 * el64 / K64, "steps": K64,
                "dtype": "f64", "fp32_speedup": v32 / v64,
                "roofline": {"bound": "fp64", "achieved": flops * K64 / el64 / 1e12,
                             "peak": peak64, "unit": "TFLOP/s",
                             "frac": flops * K64 / el64 / 1e12 / peak64,
                             "note": "nominal FFT FLOPs (5 L log2 L) per step / step time; peak "
                                     "= measured FP64 FMA throughput on this GPU"},
                "passes_ms_per_launch": dict(zip("ABC", ms64[:3]))}
        fp64.update(out.get("err", {}))
        c64.destroy()

    ensemble = None if args.no_ensemble else run_ensemble(args, torch)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(n, ps, vz, fp, fz)
    closure = None
    if rank == 0 and world == 1 and not args.no_closure:
        closure = run_closure(args.closure_small)

    line = {"metric": METRIC, "value": v32, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * el32 / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 reductions)", "data": "synthetic",
            "config": {"workload": f"single run {n}^2, RK4, dt=1e-4 fixed, nu=1e-5, hnu=0.1 (mm=2), "
                                   "Omega=10, IC k^-3 1<=|k|<=100, forcing shell 20-22",
                       "n": n, "precision": "FP32 path (headline) and FP64 path (fp64)",
                       "l2": "working set larger than L2 (6 mixed planes of 268 MB at 4096^2 FP32)",
                       "parallelism": f"replicas x{world}",
                       "plan": plan_summary(c32)},
            "gpu_launches": launches32, "roofline": roofline, "clocks": clocks, "e2e": e2e,
            "fp64": fp64, "ensemble": ensemble, "closure": closure, "cpu_baseline": cpu}
    if rank == 0:
        print(json.dumps(line), flush=True)
    c32.destroy()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
