"""Run a named workload for a number of steps on the GPU (the analogue of ``cato.x input.ini``
for the synthetic workloads), e.g. to profile one kernel on a small case:

    python -m fvleg_2d_gb300.run_case quadrant --n 2048 --precision mixed --steps 2

Workloads: ``sod`` (400x40 Sod tube), ``quadrant`` (four-quadrant Riemann problem, HLLC / van
Leer / SSP-RK3), ``kh`` (Kelvin-Helmholtz, Roe / superbee / SSP-RK3), ``circles`` (random circles,
SLAU / MLP5 / SSP-RK2, seeded), ``batch`` (the batched configuration's generator: ``--n``
instances of uneven sides in [64, 1024], random circles, SLAU / MLP5 / SSP-RK2, advanced together
in one batch).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import sys

import numpy as np

from . import ic
from .fluid import Fluid


def make(name: str, n: int, precision: str, seed: int = 0):
    if name == "sod":
        return ic.sod(precision=precision)
    if name == "quadrant":
        return ic.riemann_quadrant(n, precision=precision)
    if name == "kh":
        return ic.kelvin_helmholtz(n, precision=precision)
    if name == "circles":
        return ic.random_circles(n, n, np.random.default_rng(seed), precision=precision)
    raise ValueError(f"unknown workload {name!r}")


def run_batch(n: int, precision: str, steps: int, seed: int, plan: str, flux: str = "",
              limiter: str = "") -> dict:
    """``n`` instances of the batched configuration (seeded sides and states) in one batch;
    ``flux`` / ``limiter`` replace SLAU / MLP5 when given."""
    from .batch import Batch

    rng = np.random.default_rng(seed)
    over = {k: v for k, v in (("flux_solver", flux), ("limiter", limiter)) if v}
    insts = [ic.random_circles(nx, ny, rng, precision=precision, **over)
             for nx, ny in ic.batch_sides(n, rng)]
    b = Batch(n, precision=precision)
    if plan:
        b.set_plan(*(int(x) for x in plan.split(",")))
    for cfg, prims in insts:
        b.add(cfg, prims)
    ms = b.step(steps)
    cells = sum(c.ni * c.nj for c, _ in insts)
    b.close()
    return {"workload": "batch", "instances": n, "cells": cells, "precision": precision,
            "steps": steps, "ms": ms, "cell_updates_per_s": cells * steps / (ms / 1e3)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["sod", "quadrant", "kh", "circles", "batch"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "mixed_df"])
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--plan", default="", help="threads,rows_per_cta (default: the handle's)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="FP64 stage kernel register budget 0, 1 or 2 (default: the handle's)")
    ap.add_argument("--tune", action="store_true",
                    help="autotune plan and variant on real steps before the timed ones")
    ap.add_argument("--flux", default="", help="edge flux instead of the workload's (e.g. Roe)")
    ap.add_argument("--limiter", default="", help="limiter instead of the workload's (e.g. MLP5)")
    ap.add_argument("--t-start", type=float, default=0.0,
                    help="first advance the flow to this time with the mixed path")
    a = ap.parse_args(argv)
    if a.workload == "batch":
        print(json.dumps(run_batch(a.n, a.precision, a.steps, a.seed, a.plan, a.flux, a.limiter)))
        return 0
    cfg, prims = make(a.workload, a.n, a.precision, a.seed)
    if a.flux or a.limiter:
        old_g = cfg.ghost_layers()
        cfg = dataclasses.replace(cfg, flux_solver=a.flux or cfg.flux_solver,
                                  limiter=a.limiter or cfg.limiter)
        if cfg.ghost_layers() != old_g:  # re-pad the halo-padded primitives
            d = cfg.ghost_layers() - old_g
            prims = [np.pad(q, d, mode="edge") if d > 0 else q[-d:d, -d:d] for q in prims]
    if a.t_start > 0:
        g = Fluid(dataclasses.replace(cfg, precision="mixed")).initialize(*prims)
        g.run(a.t_start)
        s = g.state(("rho", "u", "v", "p"))
        prims = [s["rho"], s["u"], s["v"], s["p"]]
        g.close()
    f = Fluid(cfg).initialize(*prims)
    if a.plan:
        f.set_plan(*(int(x) for x in a.plan.split(",")))
    if a.variant >= 0:
        f.set_kernel_variant(a.variant)
    tuned = f.tune(2)[0] if a.tune else 0
    ms, kern = f.run_timed(a.steps, per_kernel=True)
    cells = cfg.ni * cfg.nj
    print(json.dumps({"workload": a.workload, "flux": cfg.flux_solver, "limiter": cfg.limiter,
                      "ni": cfg.ni, "nj": cfg.nj,
                      "precision": a.precision, "steps": a.steps, "ms": ms,
                      "kernel_ms": kern, "cell_updates_per_s": cells * a.steps / (ms / 1e3),
                      "plan": list(f.get_plan()), "variant": f.get_kernel_variant(),
                      "tuning_steps": tuned}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
