"""Spread independent grids over the GPUs of one node: the batched grids and the serving stream.

Both workloads shard by instance.  Grids and requests never exchange data (no halo, no global
dt, no cross-instance reduction), so each rank -- one process per GPU -- runs its own share on
its own device and the data path has no collective.  The shares are decided identically on every
rank from the same inputs, with no communication; only the per-rank totals travel, gathered over
the host process group (gloo) at the end for the whole-job figures.

* :func:`partition` -- a batch: longest-processing-time-first assignment of instances by
  predicted cost (cells x steps), each to the least-loaded rank.
* :func:`route_stream` -- a request stream: in arrival order, each request goes to the rank with
  the least predicted work assigned so far (cells x the step count a CFL time step implies).
* :func:`run_sharded` -- run this rank's share with a runner and gather every rank's totals.

The reference runs one grid per process and spreads a grid over coarray images; it has nothing
that assigns whole grids to devices.  This module is its own addition for the batched and served
configurations.
"""
from __future__ import annotations

import heapq
from typing import Callable, Sequence


def batch_cost(ni: int, nj: int, steps: int) -> float:
    """Predicted work of a batched instance: cell-updates of its fixed step count."""
    return float(ni) * float(nj) * float(steps)


def request_cost(n: int, t_end: float) -> float:
    """Predicted work of a served request on an n x n grid of [0, 1]^2 run to t_end: cells x
    steps, where the CFL step count grows as n t_end (dt proportional to the cell size)."""
    return float(n) ** 3 * float(t_end)


def partition(costs: Sequence[float], world: int) -> list[int]:
    """Rank of each item: items in decreasing cost (ties by index) go to the least-loaded rank
    (ties to the lowest rank).  Deterministic, so every rank computes the same assignment."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    owner = [0] * len(costs)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + float(costs[i]), r))
    return owner


def route_stream(costs: Sequence[float], world: int) -> list[int]:
    """Rank of each request of an arrival-ordered stream: the rank with the least predicted work
    routed to it so far (ties to the lowest rank), decided at arrival without knowing the later
    requests."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    owner = []
    for c in costs:
        r = min(range(world), key=lambda k: (load[k], k))
        owner.append(r)
        load[r] += float(c)
    return owner


def shard(owner: Sequence[int], rank: int) -> list[int]:
    """Indices owned by `rank`."""
    return [i for i, r in enumerate(owner) if r == rank]


def gather(dist, obj) -> list:
    """Every rank's object, in rank order (one rank: [obj])."""
    if dist is None:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out


def run_sharded(items: Sequence, owner: Sequence[int], rank: int, devices: Sequence[int],
                runner: Callable[[int, list], dict], dist=None) -> dict:
    """Run this rank's share and combine every rank's totals.

    ``runner(device, share)`` runs the share (a list of items) on one device and returns a dict
    with at least ``cell_updates`` and ``seconds``.  Returns the whole-job view: per-rank totals,
    ``cell_updates`` summed, ``seconds`` = the slowest rank's, and ``cell_updates_per_s``."""
    mine = [items[i] for i in shard(owner, rank)]
    local = dict(runner(devices[rank], mine))
    local.update({"rank": rank, "device": devices[rank], "items": len(mine)})
    per_rank = gather(dist, local)
    total = sum(float(r["cell_updates"]) for r in per_rank)
    slowest = max(float(r["seconds"]) for r in per_rank)
    return {"per_rank": per_rank, "cell_updates": total, "seconds": slowest,
            "cell_updates_per_s": total / slowest if slowest > 0 else None,
            "scaling": "strong (instances sharded over ranks, no collective on the data path)"}


def batch_runner(precision: str, steps: int, plan=None) -> Callable[[int, list], dict]:
    """A runner for :func:`run_sharded` that advances a share of (cfg, prims) instances in one
    batch on the given device: one persistent launch per stage, CUDA-graph chunks."""

    def run(device: int, share: list) -> dict:
        from . import _lib
        from .batch import Batch

        _lib.load().cato_gpu_select_device(int(device))
        if not share:
            return {"cell_updates": 0, "seconds": 0.0, "error_codes": []}
        b = Batch(len(share), precision=precision)
        if plan:
            b.set_plan(*plan)
        slots = [b.add(cfg, prims, max_steps=steps) for cfg, prims in share]
        ms = b.step(steps)
        qs = [b.query(s) for s in slots]
        b.close()
        return {"cell_updates": sum(q["iteration"] * c.ni * c.nj
                                    for q, (c, _) in zip(qs, share)),
                "seconds": ms / 1e3, "error_codes": [q["error_code"] for q in qs]}

    return run


def serve_runner(precision: str, budget_gb: float = 120.0,
                 max_wall_s: float = float("inf")) -> Callable[[int, list], dict]:
    """A runner for :func:`run_sharded` that serves a share of a request stream (arrival times
    kept) with the continuous-batching server on the given device."""

    def run(device: int, share: list) -> dict:
        from . import _lib
        from .serve import Server

        _lib.load().cato_gpu_select_device(int(device))
        srv = Server(precision=precision, budget_gb=budget_gb, capacity=1024)
        st = srv.serve(list(share), max_wall_s=max_wall_s)
        srv.close()
        s = st.summary()
        return {"cell_updates": s["cell_updates"], "seconds": s["wall_s"],
                "completed": s["completed"], "censored": s["censored"],
                "latencies": sorted(r.latency for r in st.completed)}

    return run


__all__ = ["batch_cost", "request_cost", "partition", "route_stream", "shard", "gather",
           "run_sharded", "batch_runner", "serve_runner"]
