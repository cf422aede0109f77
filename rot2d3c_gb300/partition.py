"""Partition of an uneven-size ensemble's runs over GPUs (one process per
GPU), and the host-side gather of their per-run diagnostics.

The reference splits ONE field over its MPI ranks in slabs (the block
partition ``range``, src/fftp.f90:17-47) and exchanges data in every
transform.  Here a single field never shards (one GPU holds the whole
plane); what shards is an ensemble of independent runs.  Runs are dealt to
ranks by their cost, n^2 log2 n per RK step (the transform work, which also
sets the memory traffic), with the longest-processing-time rule: runs in
order of decreasing cost, each to the rank with the least cost so far (ties:
the lower rank, then the lower run index), so every rank computes the same
partition without communication.  No data-path collective exists: each rank
advances its own runs, and only the per-run diagnostics (small host arrays)
are gathered at the end.
"""
from __future__ import annotations

import math


def run_cost(n: int) -> float:
    """Relative cost of one RK step of an n^2 run (n^2 log2 n)."""
    return float(n) * float(n) * math.log2(n)


def partition(ns, world: int):
    """Run indices of each rank for runs of grid sizes ``ns`` over ``world``
    ranks (LPT rule, deterministic); each rank's list is sorted."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(ns)), key=lambda i: (-run_cost(ns[i]), i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += run_cost(ns[i])
    return [sorted(p) for p in parts]


def loads(ns, parts):
    """Total cost of each rank's runs."""
    return [sum(run_cost(ns[i]) for i in p) for p in parts]


def gather_by_run(local: dict, world: int, nruns: int):
    """Host-side gather of ``{run index: diagnostics}`` from every rank into
    one list indexed by run (every rank receives it).  ``world`` = 1 needs
    no process group."""
    if world == 1:
        merged = dict(local)
    else:
        import torch.distributed as dist
        got = [None] * world
        dist.all_gather_object(got, local)
        merged = {}
        for d in got:
            for k, v in d.items():
                if k in merged:
                    raise RuntimeError(f"run {k} was advanced by two ranks")
                merged[k] = v
    missing = [i for i in range(nruns) if i not in merged]
    if missing:
        raise RuntimeError(f"runs {missing} were advanced by no rank")
    return [merged[i] for i in range(nruns)]
