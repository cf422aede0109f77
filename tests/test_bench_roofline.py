"""The roofline arithmetic of bench.py (no GPU): algorithmic bytes and
nominal FFT FLOPs per pass launch from the truncation-aware model, the
traffic read from the committed ncu summaries, and the fractions of the
line's `roofline` object."""
import math
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_algorithmic_bytes_per_launch():
    n = 4096
    L = n // 3
    M, K = L + 1, 2 * L + 1
    b32 = bench.pass_bytes(n, 4)
    assert b32["A"] == (2 * M * K + 6 * M * n) * 8      # psi, vz on M x K in; 6 mixed planes M x n out
    assert b32["B"] == (6 * M * n + 2 * M * n) * 8      # 6 planes in, 2 brackets out
    assert b32["C"] == (2 * M * n + 8 * M * K) * 8      # 2 brackets + 6 RK inputs in, c1, c2 out
    assert [round(b32[k] / 1e6) for k in "ABC"] == [328, 358, 328]
    b64 = bench.pass_bytes(n, 8)
    assert all(b64[k] == 2 * b32[k] for k in "ABC")


def test_nominal_fft_flops_per_step():
    n = 4096
    M = n // 3 + 1
    f = bench.pass_flops(n)
    per = 5.0 * n * math.log2(n)
    assert f["A"] == 6 * M * per and f["B"] == 4 * n * per and f["C"] == 2 * M * per
    # four substeps per RK4 step: 4 (8M + 4n) transforms of 5 n log2 n each
    assert 4 * sum(f.values()) == pytest.approx(26.8e9, rel=2e-3)


def test_traffic_comes_from_the_committed_capture():
    t, src = bench.pass_traffic(4096, "fp32", "B")
    assert t == 268788224 + 64605440 and src.startswith("profiles/pass_traffic_fp32_n4096.json")
    assert bench.pass_traffic(4096, "fp64", "B")[0] is not None
    assert bench.pass_traffic(123, "fp32", "B") == (None, None)


def test_roofline_object():
    n = 4096
    ms = [0.12, 0.25, 0.14, 0.0]   # ms per launch of A, B, C and the rest
    cnt = [4, 4, 4, 0]
    r = bench.roofline_of(ms, cnt, n, 4, "fp32", 6776.3, "measured")
    b = bench.pass_bytes(n, 4)
    assert r["kernel"].startswith("k_passB") and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(b["B"] / 0.25e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6776.3)
    assert r["traffic"] == 268788224 + 64605440
    assert sum(p["step_share"] for p in r["passes"].values()) == pytest.approx(1.0)
    # FP64: the FP64-pipe fraction in nominal FFT FLOPs against the measured FMA peak
    r64 = bench.roofline_of([2.56, 5.23, 1.18, 0.0], cnt, n, 8, "fp64", 6776.3, "measured", peak64=1.2546)
    fB = bench.pass_flops(n)["B"]
    assert r64["fp64_pipe"]["achieved"] == pytest.approx(fB / 5.23e-3 / 1e12)
    assert r64["fp64_pipe"]["frac"] == pytest.approx(fB / 5.23e-3 / 1e12 / 1.2546)
    assert 0.55 < r64["fp64_pipe"]["frac"] < 0.7


def _samples(t, e, inj, diss):
    import numpy as np
    S = np.zeros((len(t), 1, 30))
    S[:, 0, 0] = t
    S[:, 0, 1] = S[:, 0, 2] = e           # (E + Ez) / 2 = e
    S[:, 0, 3] = inj
    S[:, 0, 5] = diss
    return S


def test_budget_residual_closes_and_shows_the_sampling_error():
    """The ensemble leg's energy-budget residual |mean(dE/dt - (inj -
    diss))| / mean|inj|: zero for a budget that closes exactly, and, for
    an energy exchange oscillating at frequency w with a closed budget,
    small when sampled densely but large when the centred difference spans
    a sizeable part of a period (the every-tenth-step sampling)."""
    import numpy as np
    t = np.linspace(0.0, 1.0, 101)
    lin = bench.budget_residuals(_samples(t, 1.0 + 0.3 * t, np.full_like(t, 1.0), np.full_like(t, 0.7)))
    assert lin[0] == pytest.approx(0.0, abs=1e-12)
    w = 2 * np.pi * 40.0                      # a run of 0.45 periods of the exchange
    dense = np.linspace(0.0, 0.0113, 113)
    coarse = dense[::10]                      # every tenth sample
    res = []
    for tt in (dense, coarse):
        e = 1.0 + 0.05 * np.sin(w * tt)
        inj = 1.0 + 0.05 * w * np.cos(w * tt)   # inj - diss = dE/dt exactly
        res.append(bench.budget_residuals(_samples(tt, e, inj, np.full_like(tt, 1.0)))[0])
    assert res[0] < 1e-4 and res[1] > 50 * res[0]
