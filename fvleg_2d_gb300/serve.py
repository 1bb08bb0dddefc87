"""Continuous-batching serving loop over the batched engine (a stream of solve requests).

Solve requests arrive over time (Poisson arrivals in the benchmark).  The loop admits a
request as soon as a slot and enough of the HBM budget are free, keeps every admitted state on
the device, advances all running requests together in chunks of steps (each with its own dt and
t_end), and retires a request the step chunk after it finishes.  Requests that arrive while
others are on the GPU join the running batch at the next chunk boundary, and their work overlaps
with the others' on the device.  Latency = completion time - arrival time.

An instance's arithmetic does not depend on the other instances (no cross-instance reduction),
so a request's result is the same alone and in the mix (tests/test_serve_gpu.py).
"""
from __future__ import annotations

import math
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import ic
from .batch import Batch, instance_bytes
from .config import SchemeConfig

SERVING_FLUXES = ["AUSM+-up", "AUSMPW+", "SLAU", "HLLC", "Roe"]


@dataclass
class Request:
    rid: int
    arrival: float      # seconds after the stream start
    n: int              # square grid side
    flux: str
    t_end: float
    seed: int
    precision: str = "mixed"
    admitted: float = math.nan
    finished: float = math.nan
    steps: int = 0
    error_code: int = 0
    cells: int = 0
    result: dict | None = None

    def config_and_ic(self):
        rng = np.random.default_rng(self.seed)
        cfg, prims = ic.random_circles(self.n, self.n, rng, flux_solver=self.flux,
                                       limiter="minmod", integration_strategy="ssp_rk2",
                                       precision=self.precision)
        return cfg, prims

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def make_requests(n: int, rate: float, seed: int = 0, side=(128, 2048),
                  t_end=(0.05, 0.3), precision: str = "mixed") -> list[Request]:
    """The config-4 request stream: Poisson arrivals at `rate` per second, square sides
    log-uniform in `side` rounded to 16, flux uniform over the five schemes, t_end uniform."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        s = int(round(math.exp(rng.uniform(math.log(side[0]), math.log(side[1]))) / 16.0)) * 16
        out.append(Request(rid=k, arrival=t, n=max(16, s),
                           flux=SERVING_FLUXES[int(rng.integers(len(SERVING_FLUXES)))],
                           t_end=float(rng.uniform(*t_end)), seed=int(rng.integers(1 << 31)),
                           precision=precision))
    return out


@dataclass
class ServeStats:
    completed: list = field(default_factory=list)
    censored: int = 0
    wall_s: float = 0.0
    device_ms: float = 0.0
    cell_updates: int = 0

    def summary(self) -> dict:
        lat = sorted(r.latency for r in self.completed)

        def pct(p):
            if not lat:
                return None
            return lat[min(len(lat) - 1, int(math.ceil(p / 100.0 * len(lat))) - 1)]

        return {"completed": len(self.completed), "censored": self.censored,
                "ended_with_error": sum(1 for r in self.completed if r.error_code),
                "p50_latency_s": pct(50), "p99_latency_s": pct(99),
                "wall_s": self.wall_s, "device_s": self.device_ms / 1e3,
                "cell_updates": self.cell_updates,
                "cell_updates_per_s": self.cell_updates / self.wall_s if self.wall_s else None}


class Server:
    """Admission by HBM budget and slot count, device-resident state, continuous batching."""

    def __init__(self, precision: str = "mixed", budget_gb: float = 120.0, capacity: int = 512,
                 chunk_steps: int = 16, prefetch: int = 4, keep_results: bool = False):
        self.precision = precision
        self.budget = int(budget_gb * 1e9)
        self.capacity = capacity
        self.chunk = chunk_steps
        self.prefetch = prefetch
        self.keep_results = keep_results
        self.batch = Batch(capacity, precision=precision, integration_strategy="ssp_rk2")
        self.used = 0

    def close(self):
        self.batch.close()

    def serve(self, requests: list[Request], max_wall_s: float = float("inf")) -> ServeStats:
        """Run the stream; requests not finished after max_wall_s are counted as censored."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        ready: dict[int, tuple] = {}
        cv = threading.Condition()
        stop = False

        def producer():  # the clients: build each request's initial state ahead of admission
            for r in reqs:
                with cv:
                    while len(ready) >= self.prefetch and not stop:
                        cv.wait(0.05)
                    if stop:
                        return
                cfg, prims = r.config_and_ic()
                with cv:
                    ready[r.rid] = (cfg, prims)
                    cv.notify_all()

        th = threading.Thread(target=producer, daemon=True)
        th.start()
        pending = deque(reqs)
        active: dict[int, tuple[Request, int]] = {}
        stats = ServeStats()
        t0 = time.perf_counter()
        try:
            while pending or active:
                now = time.perf_counter() - t0
                if now > max_wall_s:
                    break
                # admission: arrived, IC built, a free slot and room in the HBM budget
                while pending and pending[0].arrival <= now and len(active) < self.capacity:
                    r = pending[0]
                    with cv:
                        if r.rid not in ready:
                            break
                        cfg, prims = ready[r.rid]
                    need = instance_bytes(cfg)
                    if self.used + need > self.budget and active:
                        break
                    pending.popleft()
                    with cv:
                        del ready[r.rid]
                        cv.notify_all()
                    slot = self.batch.add(cfg, prims, t_end=r.t_end)
                    r.admitted = time.perf_counter() - t0
                    r.cells = cfg.ni * cfg.nj
                    active[slot] = (r, need)
                    self.used += need
                if not active:
                    if pending:
                        time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                    continue
                stats.device_ms += self.batch.step(self.chunk)
                _, flags = self.batch.running()
                for slot, (r, need) in list(active.items()):
                    if flags[slot]:
                        continue
                    q = self.batch.query(slot)
                    r.steps, r.error_code = q["iteration"], q["error_code"]
                    if self.keep_results:
                        r.result = self.batch.state(slot)
                    r.finished = time.perf_counter() - t0
                    stats.completed.append(r)
                    stats.cell_updates += r.steps * r.cells
                    self.batch.remove(slot)
                    self.used -= need
                    del active[slot]
        finally:
            with cv:
                stop = True
                cv.notify_all()
        stats.wall_s = time.perf_counter() - t0
        stats.censored = len(pending) + len(active)
        for slot, (r, need) in active.items():
            q = self.batch.query(slot)
            stats.cell_updates += q["iteration"] * r.cells
            self.batch.remove(slot)
            self.used -= need
        return stats


def run_alone(req: Request) -> dict:
    """The same request on its own (a batch of one): the reference for the in-mix result."""
    cfg, prims = req.config_and_ic()
    b = Batch(1, precision=req.precision, integration_strategy="ssp_rk2")
    s = b.add(cfg, prims, t_end=req.t_end)
    b.run_until_done(chunk=64)
    out = b.state(s)
    q = b.query(s)
    out["steps"], out["error_code"] = q["iteration"], q["error_code"]
    b.close()
    return out


def main(argv=None) -> int:
    """Rate sweep of the request stream, one JSON line per rate:

        python -m fvleg_2d_gb300.serve --rates 10,20,50,100,200,500 --requests 200 \\
            --side 128,2048 --max-wall 30 --precision mixed
    """
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="10,20,50,100,200,500")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--side", default="128,2048")
    ap.add_argument("--t-end", default="0.05,0.3")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "mixed_df"])
    ap.add_argument("--budget-gb", type=float, default=120.0)
    ap.add_argument("--capacity", type=int, default=1024)
    ap.add_argument("--chunk", type=int, default=16)
    ap.add_argument("--max-wall", type=float, default=30.0)
    ap.add_argument("--seed", type=int, default=7)
    a = ap.parse_args(argv)
    side = tuple(int(x) for x in a.side.split(","))
    t_end = tuple(float(x) for x in a.t_end.split(","))
    for rate in (float(x) for x in a.rates.split(",")):
        reqs = make_requests(a.requests, rate=rate, seed=a.seed, side=side, t_end=t_end,
                             precision=a.precision)
        srv = Server(precision=a.precision, budget_gb=a.budget_gb, capacity=a.capacity,
                     chunk_steps=a.chunk)
        st = srv.serve(reqs, max_wall_s=a.max_wall)
        srv.close()
        out = st.summary()
        offered = sum(r.n * r.n for r in reqs if r.arrival <= st.wall_s)
        out.update({"rate_per_s": rate, "precision": a.precision, "side": list(side),
                    "arrived": sum(1 for r in reqs if r.arrival <= st.wall_s),
                    "completed_per_s": len(st.completed) / st.wall_s if st.wall_s else None,
                    "arrived_cells": offered})
        print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
