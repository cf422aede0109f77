"""Ensemble runs partitioned over ranks by cost (rot2d3c_gb300.partition):
the partition itself, and two gloo ranks on CPU that each advance their
share of a small uneven ensemble (oracle RK4 steps) and gather the per-run
diagnostics on the host, which must equal a single-rank run of all runs."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from rot2d3c_gb300 import partition as P

NS = [16, 16, 16, 16, 32, 32, 64]


def test_partition_covers_every_run_once_and_balances_cost():
    for world in (1, 2, 3, 4):
        parts = P.partition(NS, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(NS)))
        ld = P.loads(NS, parts)
        # LPT: no rank exceeds the mean load by more than the largest run
        assert max(ld) <= sum(ld) / world + max(P.run_cost(n) for n in NS) + 1e-9
    assert P.partition(NS, 2) == P.partition(list(NS), 2)  # deterministic
    # the config-3 ensemble on 8 ranks: 64 x 512^2 + 16 x 1024^2 + 4 x 2048^2
    big = [512] * 64 + [1024] * 16 + [2048] * 4
    ld = P.loads(big, P.partition(big, 8))
    assert max(ld) / (sum(ld) / 8) < 1.05


def _run_diagnostics(i):
    """Three oracle RK4 steps of run i; its energies and energy spectrum."""
    from oracle import rot2d3c_oracle as O
    from tests._helpers import random_forcing, random_state
    n = NS[i]
    g, ps, vz = random_state(n, 100 + i, kmax_shell=n / 4.0)
    fp, fz = random_forcing(g, 200 + i, 2.0, 3.0)
    p = O.Params(n=n, omega=0.5 * (i + 1), nu=1e-3, nuv=1e-3, hnu=0.1, hnuv=0.1, iflow=0)
    for _ in range(3):
        ps, vz, fp, fz = O.rk_step(g, p, ps, vz, fp, fz, 1e-3)
    ek, ezk = O.spectrum(g, ps, vz)
    return {"n": n, "e": O.energy(g, ps, 1), "ez": O.energy(g, vz, 0), "ek": ek.tolist()}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from rot2d3c_gb300 import partition as Pw
    mine = Pw.partition(NS, world)[rank]
    local = {i: _run_diagnostics(i) for i in mine}
    allruns = Pw.gather_by_run(local, world, len(NS))
    q.put((rank, mine, allruns))
    dist.destroy_process_group()


def test_two_ranks_gather_the_single_rank_diagnostics():
    want = P.gather_by_run({i: _run_diagnostics(i) for i in range(len(NS))}, 1, len(NS))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (r0, m0, g0), (r1, m1, g1) = res
    assert sorted(m0 + m1) == list(range(len(NS))) and not set(m0) & set(m1)
    for got in (g0, g1):
        assert len(got) == len(NS)
        for a, b in zip(got, want):
            assert a["n"] == b["n"] and a["e"] == b["e"] and a["ez"] == b["ez"]
            np.testing.assert_array_equal(a["ek"], b["ek"])


def test_gather_refuses_a_missing_run():
    with pytest.raises(RuntimeError):
        P.gather_by_run({0: 1.0}, 1, 2)
