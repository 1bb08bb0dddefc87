#!/usr/bin/env python
"""Benchmark of the GB300 time-step hot path: cell-updates/s on the 4096x4096 four-quadrant
Riemann problem (HLLC flux, van Leer limiter, SSP-RK3, CFL 0.4, transmissive boundaries).

A "step" is one full SSP-RK3 time step (three fused stage kernels + the step-control kernel) of
the whole grid; value = cell-updates/s of the plain FP64 path with the state resident in HBM.
The mixed path (FP32 reconstruction/flux, FP64 state) is reported beside it, and e2e measures
the same metric through the C-ABI with host buffers (upload + per-step cato_gpu_integrate +
download inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (torchrun): one independent replica per GPU ("replicas only": the grid is not split),
value = sum of the replicas' cell-updates over the slowest replica's time.
--impl reference: the CPU restatement of the reference (C, OpenMP on all host cores) on the same
grid and scheme; rank 0 only.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s & HBM GB/s, plain FP64 vs mixed/batched; p99 solve latency"
HBM_FALLBACK_GBS = 6800.0
# algorithmic HBM bytes per cell and stage kernel launch (state in, state out), SSP-RK3, the same
# FP64 state layout in every precision: stage 1 reads U^n and writes U1 (64 B); stages 2 and 3
# read U^n and U^k and write 32 B (96 B)
BYTES_PER_CELL_STAGE = {"fp64": (64, 96, 96), "mixed": (64, 96, 96), "mixed_df": (64, 96, 96)}


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            with open(path) as f:
                d = json.load(f)
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return HBM_FALLBACK_GBS, "fallback"


def profile_traffic():
    """Per-cell DRAM bytes of the stage kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clocks during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def dist_setup():
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch.distributed as dist  # host-side barrier / max only (gloo, CPU tensors)

        dist.init_process_group("gloo")
    return world, rank, local, dist


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_reference(cfg, prims, steps: int, warmup: int, threads: int):
    """The C oracle (restatement of the reference) on `steps` full time steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    used = O.set_threads(threads)
    f = O.OracleFluid(cfg)
    f.set_primitive(*prims)
    for _ in range(warmup):
        f.integrate()
    t0 = time.perf_counter()
    for _ in range(steps):
        ec = f.integrate()
        if ec:
            raise RuntimeError(f"oracle error code {ec}")
    dt = time.perf_counter() - t0
    return cfg.ni * cfg.nj * steps / dt, used, dt


def run_reference(args, world, rank, dist):
    if rank != 0:
        return 0
    from fvleg_2d_gb300 import ic

    cfg, prims = ic.riemann_quadrant(args.n)
    threads = os.cpu_count() or 1
    value, used, secs = cpu_reference(cfg, prims, args.steps, args.warmup, threads)
    sample = (f"{args.steps} SSP-RK3 steps of the {args.n}x{args.n} grid after {args.warmup} "
              f"warm-up steps ({secs:.1f} s)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload_config(args, world),
                       window="steps from the initial state, not the GPU arm's developed window "
                              "at t = 0.15: reaching it takes ~1100 steps of the 4096^2 grid, "
                              "hours of this CPU arm; the restatement has no data-dependent "
                              "shortcuts, and the GPU arm's cpu_baseline times it on the "
                              "developed state itself",
                       same_window=False),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": used,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, world):
    return {"workload": f"four-quadrant 2-D Riemann problem {args.n}x{args.n} over [0,1]^2",
            "flux": "HLLC", "limiter": "van_leer", "integrator": "ssp_rk3", "cfl": 0.4,
            "gamma": 1.4, "bc": "zero_gradient (transmissive) on all sides",
            "cells": args.n * args.n, "n_ghost": 2,
            "l2": "state of 4 x 8 B x 16.8M cells = 537 MB per copy > 129 MB L2 (no flush needed)",
            "window": (f"steps from the developed flow at t = {args.t_start} (state advanced with "
                       "the mixed path, then uploaded as primitives)" if args.t_start > 0
                       else "steps from the initial state"),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


_DEVELOPED = {}


def quadrant_state(args):
    """The quadrant problem's state at t = args.t_start (primitives, halo-padded): the timed
    window is taken from the developed flow rather than from the piecewise-constant initial
    state, whose uniform regions make every path's data-dependent shortcuts unrepresentatively
    cheap.  The state is advanced with the mixed path (its accuracy is irrelevant to a
    throughput window) and cached for all legs."""
    from fvleg_2d_gb300 import ic
    from fvleg_2d_gb300.fluid import Fluid

    key = (args.n, args.t_start)
    # optional on-disk copy (CATO_BENCH_STATE_CACHE=<dir>), so that a profiler run of the bench
    # after a plain run does not spend its launch budget on the mixed-path advance
    cache_dir = os.environ.get("CATO_BENCH_STATE_CACHE")
    cache = (os.path.join(cache_dir, f"quadrant_{args.n}_{args.t_start}.npz")
             if cache_dir and args.t_start > 0 else None)
    if key not in _DEVELOPED and cache and os.path.exists(cache):
        import numpy as np

        cfg, _ = ic.riemann_quadrant(args.n)
        with np.load(cache) as z:
            _DEVELOPED[key] = (cfg, [np.asfortranarray(z[k]) for k in ("rho", "u", "v", "p")])
    if key not in _DEVELOPED:
        cfg, prims = ic.riemann_quadrant(args.n)
        if args.t_start > 0:
            f = Fluid(dataclasses.replace(cfg, precision="mixed")).initialize(*prims)
            f.run(args.t_start)
            s = f.state(("rho", "u", "v", "p"))
            prims = [s["rho"], s["u"], s["v"], s["p"]]
            f.close()
            if cache:
                import numpy as np

                os.makedirs(cache_dir, exist_ok=True)
                np.savez(cache, **dict(zip(("rho", "u", "v", "p"), prims)))
        _DEVELOPED[key] = (cfg, prims)
    return _DEVELOPED[key]


def bench_precision(args, precision, dist, world, peak_gbs):
    from fvleg_2d_gb300.fluid import Fluid

    cfg, prims = quadrant_state(args)
    cfg = dataclasses.replace(cfg, precision=precision)
    f = Fluid(cfg).initialize(*prims)
    tuned_steps, _ = f.tune(2)  # plan and kernel variant, on real steps before the warm-up
    f.run_timed(args.warmup)
    barrier(dist)
    with ClockSampler(env_int("LOCAL_RANK", 0)) as clk:
        total_ms, kernel_ms = f.run_timed(args.steps, per_kernel=True)
    barrier(dist)
    max_ms = allreduce_max(dist, total_ms)
    cells = cfg.ni * cfg.nj
    value = world * cells * args.steps / (max_ms / 1000.0)
    per_stage = BYTES_PER_CELL_STAGE[precision]
    stage_ms = kernel_ms[1:]
    stage_bytes = sum(per_stage) * cells * args.steps
    achieved = stage_bytes / (sum(stage_ms) / 1000.0) / 1e9
    n_stage_launches = len(per_stage) * args.steps
    traffic = profile_traffic().get(f"{precision}_stage_bytes_per_cell")
    res = {
        "value": value,
        "ms_per_step": max_ms / args.steps,
        "launches_per_step": f.launches_per_step(),
        "stage_ms_per_step": [m / args.steps for m in stage_ms],
        "step_control_ms_per_step": kernel_ms[0] / args.steps,
        "roofline": {
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak_gbs,
            "unit": "GB/s",
            "frac": achieved / peak_gbs,
            "traffic": (traffic * cells if traffic else None),
            "algorithmic_bytes_per_launch": stage_bytes / n_stage_launches,
        },
        "clocks": clk.summary(),
        "plan": {"threads": f.get_plan()[0], "rows_per_cta": f.get_plan()[1],
                 "kernel_variant": f.get_kernel_variant(), "tuning_steps": tuned_steps},
    }
    if precision == "fp64":
        # The FP64 kernel is bound by GB300's FP64 pipe (2 FP64 thread-instructions per SM and
        # cycle), not by HBM: FP64-pipe instructions per cell and stage from the ncu capture of
        # the same kernel on the developed flow, over the stage time, against 2 x SMs x the SM
        # clock sampled during the timed region.
        ipc = profile_traffic().get("fp64_pipe_inst_per_cell_stage")
        mhz = res["clocks"].get("sm_mhz") or res["clocks"].get("sm_max_mhz")
        if ipc and mhz:
            sms = _sm_count()
            got = ipc * cells * len(per_stage) * args.steps / (sum(stage_ms) / 1e3) / 1e9
            peak = 2 * sms * mhz / 1e3
            res["roofline"]["fp64_pipe"] = {
                "achieved": got, "peak": peak, "unit": "G FP64 thread-instructions/s",
                "frac": got / peak, "instructions_per_cell_stage": ipc}
    f.close()
    return res, cfg, prims


def _sm_count() -> int:
    try:
        import torch

        return torch.cuda.get_device_properties(env_int("LOCAL_RANK", 0)).multi_processor_count
    except Exception:
        return 152


def bench_e2e(args, cfg, prims, plan):
    """Through the C-ABI with pinned host buffers: upload, per-step integrate (dt and error code
    back to the host each step), download of the final conserved state.  The handle runs the
    plan the device-timed leg of the same precision tuned (a second tuning on two steps per
    candidate picks a slower plan now and then)."""
    import ctypes

    from fvleg_2d_gb300 import _lib
    from fvleg_2d_gb300.fluid import Fluid

    pinned = [_lib.PinnedArray(cfg.halo_shape) for _ in range(8)]
    for k in range(4):
        pinned[k].array[...] = prims[k]
    f = Fluid(cfg)
    # warm-up on the same handle (allocations, module load)
    f.initialize(*(p.array for p in pinned[:4]))
    f.set_plan(plan["threads"], plan["rows_per_cta"])
    f.set_kernel_variant(plan["kernel_variant"])
    for _ in range(min(args.warmup, 2)):
        f.integrate()
    L, h, ld = f.L, f.h, f.ld
    used, ec = ctypes.c_double(), ctypes.c_int32()
    # the sequence restarts from the same upload each time: the median of three runs (one run
    # of the host-clocked sequence now and then catches a host-side stall)
    runs = []
    for _ in range(3):
        t0 = time.perf_counter()
        rc = L.cato_gpu_upload_primitive(h, *(_lib.ptr(p.array) for p in pinned[:4]), ld)
        for _ in range(args.steps):
            rc |= L.cato_gpu_integrate(h, 0.0, ctypes.byref(used), ctypes.byref(ec))
        rc |= L.cato_gpu_download(h, *(_lib.ptr(p.array) for p in pinned[4:8]), None, None,
                                  None, None, ld)
        runs.append(time.perf_counter() - t0)
        if rc or ec.value:
            raise RuntimeError(f"e2e run failed rc={rc} ec={ec.value}")
    secs = sorted(runs)[1]
    f.close()
    for p in pinned:
        p.free()
    cells = cfg.ni * cfg.nj
    state_bytes = 4 * cells * 8
    ctl = 72  # step-control block each way per integrate call
    return {"value": cells * args.steps / secs, "unit": "cell-updates/s",
            "h2d_bytes_per_step": state_bytes / args.steps + ctl,
            "d2h_bytes_per_step": state_bytes / args.steps + 2 * ctl,
            "sequence": "upload_primitive + K x integrate + download (pinned host buffers); "
                        "median of 3 runs of the sequence"}


def bench_kh(args, peak_gbs):
    """Roofline stress: Kelvin-Helmholtz shear layer on 8192^2 (Roe with Harten's entropy fix,
    superbee, SSP-RK3, CFL 0.4, periodic x, symmetry y).  The mixed path runs the full 200-step
    window from the initial state; the double-float and FP64 paths then time a window of steps
    from the state the mixed run reached (the developed shear layer, uploaded as primitives).
    Each handle is autotuned on a few real steps first."""
    from fvleg_2d_gb300 import ic
    from fvleg_2d_gb300.fluid import Fluid

    out = {}
    developed = None
    for precision, steps in (("mixed", args.kh_steps), ("mixed_df", args.kh_df_steps),
                             ("fp64", args.kh_fp64_steps)):
        if steps <= 0:
            continue
        cfg, prims = ic.kelvin_helmholtz(args.kh_n, roe_entropy_fix="harten", precision=precision)
        start = "initial state"
        if precision != "mixed" and developed is not None:
            prims, start = developed
        f = Fluid(cfg).initialize(*prims)
        f.tune(1 if precision == "fp64" else 2)
        f.run_timed(3)
        with ClockSampler(env_int("LOCAL_RANK", 0)) as clk:
            total_ms, kernel_ms = f.run_timed(steps, per_kernel=True)
        if precision == "mixed":
            s = f.state(("rho", "u", "v", "p"))
            developed = ([s["rho"], s["u"], s["v"], s["p"]],
                         f"developed state at t = {f.time:.4f} after the mixed window")
        cells = cfg.ni * cfg.nj
        per_stage = BYTES_PER_CELL_STAGE[precision]
        achieved = sum(per_stage) * cells * steps / (sum(kernel_ms[1:]) / 1e3) / 1e9
        out[precision] = {
            "value": cells * steps / (total_ms / 1e3), "unit": "cell-updates/s",
            "steps": steps, "ms_per_step": total_ms / steps, "window_start": start,
            "plan": {"threads": f.get_plan()[0], "rows_per_cta": f.get_plan()[1],
                     "kernel_variant": f.get_kernel_variant()},
            "stage_ms_per_step": [m / steps for m in kernel_ms[1:]],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                         "frac": achieved / peak_gbs,
                         "algorithmic_bytes_per_cell_update": sum(per_stage)},
            "clocks": clk.summary(),
        }
        f.close()
    out["workload"] = (f"Kelvin-Helmholtz {args.kh_n}x{args.kh_n}, Roe + Harten, superbee, "
                       "SSP-RK3, CFL 0.4, periodic x / symmetry y; 3 warm-up steps")
    return out


def layered_grid_nodes(n: int) -> tuple:
    """Interior nodes of an n x n pycato-style grid on [0,1]^2: x in three constant-spacing
    layers (n/8 cells over 0.05, n/4 over 0.2, the rest over 0.75, stitched like
    make_2d_layered_grid), y from numpy.linspace (make_uniform_grid)."""
    import numpy as np

    counts = (n // 8, n // 4, n - n // 8 - n // 4)
    parts, start = [], 0.0
    for thickness, count in zip((0.05, 0.2, 0.75), counts):
        parts.append(np.linspace(start, start + thickness, count + 1))
        start += thickness
    return np.unique(np.concatenate(parts)), np.linspace(0.0, 1.0, n + 1)


def bench_rectilinear(args, uniform_values):
    """The rectilinear-grid path (per-column / per-row metrics, per-cell volume and division):
    the developed quadrant state on a layered n x n grid, each precision against its
    uniform-grid value."""
    from fvleg_2d_gb300.fluid import Fluid

    cfg0, prims = quadrant_state(args)
    xs, ys = layered_grid_nodes(args.n)
    out = {"workload": (f"developed quadrant state on a {args.n}x{args.n} layered grid "
                        "(x: 3 constant-spacing layers, cell widths 1 : 2 : 3, y: linspace)")}
    for precision in ("fp64", "mixed", "mixed_df"):
        cfg = dataclasses.replace(cfg0, precision=precision)
        f = Fluid(cfg).set_rectilinear(xs, ys).initialize(*prims)
        f.tune(2)
        f.run_timed(args.warmup)
        with ClockSampler(env_int("LOCAL_RANK", 0)) as clk:
            total_ms, _ = f.run_timed(args.steps, per_kernel=False)
        value = cfg.ni * cfg.nj * args.steps / (total_ms / 1e3)
        out[precision] = {"value": value, "unit": "cell-updates/s",
                          "ms_per_step": total_ms / args.steps,
                          "plan": {"threads": f.get_plan()[0], "rows_per_cta": f.get_plan()[1],
                                   "kernel_variant": f.get_kernel_variant()},
                          "vs_uniform_grid": value / uniform_values[precision],
                          "clocks": clk.summary()}
        f.close()
    return out


def bench_slabs(args, one_grid):
    """The developed quadrant grid split into 2 row slabs on this one GPU (fvleg_2d_gb300.slabs):
    each stage waits for the edge rows of both slabs to pass through the host, as a
    multi-GPU run would exchange them between processes.  Timed on the host clock (every stage
    synchronises), against the one-grid value of the same precision and plan."""
    import time

    from fvleg_2d_gb300 import slabs
    from fvleg_2d_gb300.fluid import Fluid

    cfg0, prims = quadrant_state(args)
    world = 2
    out = {"workload": f"developed quadrant state, {args.n}x{args.n}, 2 row slabs on one GPU "
                       "(host-staged edge-row exchange before every stage)"}
    for precision in ("fp64", "mixed"):
        cfg = dataclasses.replace(cfg0, precision=precision)
        parts = [slabs.slab_config(cfg, r, world) for r in range(world)]
        fluids = [Fluid(c).initialize(*slabs.slab_fields(cfg, prims, j0, j1))
                  for c, j0, j1 in parts]
        plan = one_grid[precision]["plan"]
        for f in fluids:
            f.set_plan(plan["threads"], plan["rows_per_cta"])
            f.set_kernel_variant(plan["kernel_variant"])
        run = slabs.SlabRun(fluids, slabs.SlabComm(world, False))
        for _ in range(args.warmup):
            run.step()
        with ClockSampler(env_int("LOCAL_RANK", 0)) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                run.step()
            secs = time.perf_counter() - t0
        value = cfg.ni * cfg.nj * args.steps / secs
        g = cfg.ghost_layers()
        out[precision] = {"value": value, "unit": "cell-updates/s",
                          "ms_per_step": secs * 1e3 / args.steps,
                          "vs_one_grid": value / one_grid[precision]["value"],
                          "exchange_bytes_per_stage": 2 * 2 * 4 * g * cfg.ni * 8,
                          "clocks": clk.summary()}
        for f in fluids:
            f.close()
    return out


def error_stats(x):
    """Median, p90, p99, max and the count above 1e-6 of a list of per-instance errors."""
    import numpy as np

    if not x:
        return {"n": 0}
    a = np.asarray(x, dtype=np.float64)
    return {"n": int(a.size), "median": float(np.median(a)),
            "p90": float(np.quantile(a, 0.90)), "p99": float(np.quantile(a, 0.99)),
            "max": float(a.max()), "above_1e-6": int((a > 1e-6).sum())}


def fp64_conditioning(insts, ref, rhos, codes, steps, worst=8):
    """How far the FP64 run itself moves when its initial state is perturbed by 1e-13 (relative,
    per cell), for the instances where the double-float path is furthest from FP64: an instance
    whose flow amplifies a 1e-13 perturbation beyond 1e-6 cannot be held within 1e-6 of FP64 by
    any arithmetic that is not bit-identical to it."""
    import numpy as np

    from fvleg_2d_gb300.batch import Batch

    errs = []
    for i in range(len(insts)):
        if ref[0][i] or codes[i]:
            continue
        a = ref[1][i]
        errs.append((float(np.abs(rhos[i] - a).sum() / np.abs(a).sum()), i))
    pick = [i for e, i in sorted(errs, reverse=True)[:worst]]
    if not pick:
        return None
    prng = np.random.default_rng(5)
    b = Batch(len(pick), precision="fp64")
    slots = []
    for i in pick:
        cfg, prims = insts[i]
        p = [q.copy(order="F") for q in prims]
        for q in p:
            q *= 1.0 + 1e-13 * prng.standard_normal(q.shape)
        slots.append(b.add(cfg, p, max_steps=steps))
    b.step(steps)
    rows = []
    for i, s in zip(pick, slots):
        g = insts[i][0].ghost_layers()
        r = b.state(s)["rho"][g:-g, g:-g]
        a = ref[1][i]
        rows.append({"instance": i, "ni": insts[i][0].ni, "nj": insts[i][0].nj,
                     "mixed_df_rel_l1": float(np.abs(rhos[i] - a).sum() / np.abs(a).sum()),
                     "fp64_perturbed_1e-13_rel_l1": float(np.abs(r - a).sum() / np.abs(a).sum()),
                     "perturbed_code": b.query(s)["error_code"]})
    b.close()
    return {"perturbation": "FP64 initial state x (1 + 1e-13 N(0,1)) per cell", "instances": rows}


def bench_batched(args):
    """Config 3: 256 uneven grids (sides log-uniform [64,1024] rounded to 16, aspect U[1,4]),
    random circles, SLAU + MLP5, SSP-RK2, CFL 0.5, 500 steps each; one persistent launch per
    stage, CUDA-graph chunks, autotuned tile plan.  Timed in FP64 (the plain path on the same
    workload) and in the two mixed precisions; every instance's final density is compared with
    its FP64 result (relative L1 and Linf over all instances that finish in both), and every
    instance's error code with its FP64 code."""
    import numpy as np

    from fvleg_2d_gb300 import ic
    from fvleg_2d_gb300.batch import Batch

    rng = np.random.default_rng(args.batch_seed)
    sides = ic.batch_sides(args.batch_n, rng)
    insts = [ic.random_circles(nx, ny, rng) for nx, ny in sides]
    cells = sum(c.ni * c.nj for c, _ in insts)
    precisions = args.batch_precisions.split(",")
    if "fp64" in precisions:  # the reference of the error statistics runs first
        precisions = ["fp64"] + [p for p in precisions if p != "fp64"]
    ref = None
    out = {}
    for precision in precisions:
        pinsts = [(dataclasses.replace(c, precision=precision), p) for c, p in insts]
        # autotune the shared tile plan on a scratch batch of the same instances
        tune = Batch(len(pinsts), precision=precision)
        for cfg, prims in pinsts:
            tune.add(cfg, prims)
        table = {}
        for threads, rows in [(64, 16), (128, 16), (128, 32), (256, 16), (256, 32)]:
            tune.set_plan(threads, rows)
            tune.step(2)
            table[f"{threads}x{rows}"] = tune.step(4) / 4
        tune.close()
        best = min(table, key=table.get)
        threads, rows = (int(x) for x in best.split("x"))
        b = Batch(len(pinsts), precision=precision)
        b.set_plan(threads, rows)
        slots = [b.add(cfg, prims, max_steps=args.batch_steps) for cfg, prims in pinsts]
        ms = b.step(args.batch_steps)
        n_run, _ = b.running()
        qs = [b.query(s) for s in slots]
        codes = [q["error_code"] for q in qs]
        updates_done = sum(q["iteration"] * c.ni * c.nj for q, (c, _) in zip(qs, pinsts))
        value = updates_done / (ms / 1e3)
        rhos = []
        for i, s in enumerate(slots):
            g = insts[i][0].ghost_layers()
            rhos.append(b.state(s)["rho"][g:-g, g:-g].copy())
        b.close()
        # algorithmic bytes per cell-update, SSP-RK2 on the FP64 state layout: 64 + 96
        res = {
            "value": value, "unit": "cell-updates/s", "device_ms": ms, "still_running": n_run,
            "ended_with_error": sum(1 for c in codes if c), "cell_updates": updates_done,
            "plan": {"threads": threads, "rows_per_cta": rows, "tuning_ms_per_step": table},
            "roofline": {"bound": "hbm", "achieved": value * 160 / 1e9, "unit": "GB/s",
                         "algorithmic_bytes_per_cell_update": 160},
        }
        if precision == "fp64":
            ref = (codes, rhos)
        elif ref is not None:
            l1, linf = [], []
            for i in range(len(insts)):
                if ref[0][i] or codes[i]:
                    continue
                a, m = ref[1][i], rhos[i]
                l1.append(float(np.abs(m - a).sum() / np.abs(a).sum()))
                linf.append(float(np.abs(m - a).max() / np.abs(a).max()))
            diff = [(i, ref[0][i], codes[i]) for i in range(len(insts)) if ref[0][i] != codes[i]]
            res["density_error_vs_fp64"] = {"rel_l1": error_stats(l1),
                                            "rel_linf": error_stats(linf),
                                            "instances_compared": len(l1)}
            res["error_codes_vs_fp64"] = {"agree": len(insts) - len(diff),
                                          "disagree_instance_fp64_this": [list(t) for t in diff]}
            if "fp64" in out:
                res["speedup_vs_fp64_batched"] = value / out["fp64"]["value"]
            if precision == "mixed_df":
                res["conditioning"] = fp64_conditioning(insts, ref, rhos, codes, args.batch_steps)
        out[precision] = res
    out.update({
        "instances": len(insts), "cells": cells, "steps_each": args.batch_steps,
        "launches_per_step": 4,
        "scheme": "SLAU, MLP5 (3 ghost layers), SSP-RK2, CFL 0.5, zero-gradient BCs",
        "precisions": {"fp64": "FP64 reconstruction/flux (the plain path), FP64 state",
                       "mixed": "FP32 reconstruction/flux/divergence, FP64 stage accumulation",
                       "mixed_df": "double-float (FP32 pairs) reconstruction/flux/divergence, "
                                   "FP64 stage accumulation"},
    })
    return out


def bench_batched_sharded(args, rank, world, local, dist):
    """Config 3 over several GPUs: the instances shard by predicted work (longest first, each to
    the least-loaded rank) and every rank advances its share in one batch on its own GPU; no
    collective on the data path, only the per-rank totals are gathered.  Whole-job throughput =
    all ranks' cell-updates / the slowest rank's device time."""
    import numpy as np

    from fvleg_2d_gb300 import dispatch, ic

    rng = np.random.default_rng(args.batch_seed)
    sides = ic.batch_sides(args.batch_n, rng)
    insts = [ic.random_circles(nx, ny, rng) for nx, ny in sides]
    owner = dispatch.partition([dispatch.batch_cost(c.ni, c.nj, args.batch_steps)
                                for c, _ in insts], world)
    out = {}
    for precision in args.batch_precisions.split(","):
        pinsts = [(dataclasses.replace(c, precision=precision), p) for c, p in insts]
        res = dispatch.run_sharded(pinsts, owner, rank, list(range(world)),
                                   dispatch.batch_runner(precision, args.batch_steps, (256, 32)),
                                   dist)
        out[precision] = {"value": res["cell_updates_per_s"], "unit": "cell-updates/s",
                          "slowest_rank_s": res["seconds"],
                          "per_rank": [{k: r[k] for k in ("rank", "items", "cell_updates",
                                                          "seconds")} for r in res["per_rank"]],
                          "scaling": res["scaling"]}
    out.update({"instances": len(insts), "steps_each": args.batch_steps, "ranks": world,
                "scheme": "SLAU, MLP5 (3 ghost layers), SSP-RK2, CFL 0.5, zero-gradient BCs"})
    return out


def bench_serving(args):
    """Config 4: a Poisson stream of solve requests (square sides log-uniform in [128, 2048],
    random-circle states, flux uniform over AUSM+-up, AUSMPW+, SLAU, HLLC and Roe, minmod,
    SSP-RK2, CFL 0.5, t_end U[0.05, 0.3]) through the continuous-batching server with a 120 GB
    HBM admission budget, at several arrival rates and in every precision.  Each stream is cut
    after a wall-time cap: requests still queued or running then are censored.  A mean request
    is ~1e9-1e10 cell-updates, so the offered load exceeds the GPU at every rate of the sweep and
    the sustainable request rate is what completes within the cap."""
    from fvleg_2d_gb300.serve import Server, make_requests

    out = {}
    rates = [float(x) for x in args.serve_rates.split(",")]
    for precision in ("mixed", "mixed_df", "fp64"):
        rows = []
        for rate in rates:
            reqs = make_requests(args.serve_n, rate=rate, seed=args.serve_seed,
                                 side=(args.serve_min_side, args.serve_max_side),
                                 precision=precision)
            srv = Server(precision=precision, budget_gb=120.0, capacity=1024, chunk_steps=16)
            st = srv.serve(reqs, max_wall_s=args.serve_max_wall)
            srv.close()
            row = st.summary()
            row.update({"rate_per_s": rate,
                        "arrived": sum(1 for r in reqs if r.arrival <= st.wall_s),
                        "sustained_req_per_s": (row["completed"] / st.wall_s
                                                if st.wall_s else None)})
            rows.append(row)
        out[precision] = rows
    out["stream"] = {"requests": args.serve_n, "rates_per_s": rates,
                     "side": [args.serve_min_side, args.serve_max_side], "t_end": [0.05, 0.3],
                     "fluxes": "AUSM+-up, AUSMPW+, SLAU, HLLC, Roe (uniform)",
                     "scheme": "minmod, SSP-RK2, CFL 0.5, zero-gradient BCs",
                     "admission": "120 GB HBM budget", "wall_cap_s": args.serve_max_wall}
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--t-start", type=float, default=0.15,
                    help="start the timed window from the quadrant flow at this time")
    ap.add_argument("--cpu-baseline-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-n", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--batch-seed", type=int, default=2024)
    ap.add_argument("--batch-precisions", default="fp64,mixed_df,mixed")
    ap.add_argument("--no-rectilinear", action="store_true")
    ap.add_argument("--no-kh", action="store_true")
    ap.add_argument("--no-slabs", action="store_true")
    ap.add_argument("--kh-n", type=int, default=8192)
    ap.add_argument("--kh-steps", type=int, default=200)
    ap.add_argument("--kh-fp64-steps", type=int, default=20)
    ap.add_argument("--kh-df-steps", type=int, default=20)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-n", type=int, default=2000)
    ap.add_argument("--serve-rates", default="10,100,500")
    ap.add_argument("--serve-seed", type=int, default=7)
    ap.add_argument("--serve-min-side", type=int, default=128)
    ap.add_argument("--serve-max-side", type=int, default=2048)
    ap.add_argument("--serve-max-wall", type=float, default=10.0)
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank, dist)

    from fvleg_2d_gb300 import _lib

    _lib.load(build_if_missing=True).cato_gpu_select_device(local)
    peak, peak_kind = measured_peaks()
    fp64, cfg, prims = bench_precision(args, "fp64", dist, world, peak)
    mixed, _, _ = bench_precision(args, "mixed", dist, world, peak)
    mixed_df, _, _ = bench_precision(args, "mixed_df", dist, world, peak)
    plans = {"fp64": fp64["plan"], "mixed": mixed["plan"], "mixed_df": mixed_df["plan"]}

    def e2e_of(precision):
        c = dataclasses.replace(cfg, precision=precision)
        r = bench_e2e(args, c, prims, plans[precision])
        r["value"] = -allreduce_max(dist, -r["value"]) * world  # slowest replica
        return r

    e2e = e2e_of("fp64")
    e2e_mixed = e2e_of("mixed")
    e2e_df = e2e_of("mixed_df")
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, used, secs = cpu_reference(cfg, prims, args.cpu_baseline_steps, 0, threads)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": used, "kind": "port",
               "sample": f"{args.cpu_baseline_steps} SSP-RK3 steps of the same {args.n}^2 grid "
                         f"({secs:.1f} s, OpenMP C restatement of the reference)"}
    rect = None if args.no_rectilinear else bench_rectilinear(
        args, {"fp64": fp64["value"], "mixed": mixed["value"], "mixed_df": mixed_df["value"]})
    kh = None if args.no_kh else bench_kh(args, peak)
    slab = None if args.no_slabs else bench_slabs(args, {"fp64": fp64, "mixed": mixed})
    if args.no_batched:
        batched = None
    elif world > 1:
        batched = bench_batched_sharded(args, rank, world, local, dist)
    else:
        batched = bench_batched(args)
    serving = None if args.no_serving else bench_serving(args)
    if rank != 0:
        return 0
    launches = fp64["launches_per_step"] * args.steps
    line = {
        "metric": METRIC,
        "value": fp64["value"],
        "unit": "cell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": fp64["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": dict(workload_config(args, world), plan=fp64["plan"]),
        "hbm_gbs": fp64["roofline"]["achieved"],
        "roofline": dict(fp64["roofline"], peak_source=f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                         if peak_kind == "measured" else "fallback 6.8 TB/s"),
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": fp64["clocks"],
        "stage_ms_per_step": fp64["stage_ms_per_step"],
        "mixed": {
            "value": mixed["value"], "unit": "cell-updates/s", "dtype": "f32 reconstruction/flux, f64 stage accumulation",
            "ms_per_step": mixed["ms_per_step"], "speedup_vs_fp64": mixed["value"] / fp64["value"],
            "roofline": mixed["roofline"], "stage_ms_per_step": mixed["stage_ms_per_step"],
            "gpu_launches": mixed["launches_per_step"] * args.steps, "clocks": mixed["clocks"],
            "plan": mixed["plan"], "e2e": e2e_mixed,
        },
        "mixed_df": {
            "value": mixed_df["value"], "unit": "cell-updates/s",
            "dtype": "double-float (FP32 pairs) flux / f64 state",
            "ms_per_step": mixed_df["ms_per_step"],
            "speedup_vs_fp64": mixed_df["value"] / fp64["value"],
            "roofline": mixed_df["roofline"], "stage_ms_per_step": mixed_df["stage_ms_per_step"],
            "gpu_launches": mixed_df["launches_per_step"] * args.steps,
            "clocks": mixed_df["clocks"], "plan": mixed_df["plan"], "e2e": e2e_df,
        },
        "rectilinear": rect,
        "slabs": slab,
        "kelvin_helmholtz": kh,
        "batched": batched,
        "serving": serving,
    }
    try:  # last, so that a tail of the line shows every leg
        line["summary"] = summary_of(line)
    except (KeyError, TypeError) as exc:
        line["summary"] = {"unavailable": repr(exc)}
    print(json.dumps(line), flush=True)
    return 0


def summary_of(line: dict) -> dict:
    """The figures of every leg in one short object (cell-updates/s in G, errors, latencies)."""
    def g(v):
        return None if v is None else round(v / 1e9, 4)

    out = {"unit": "G cell-updates/s",
           "quadrant": {"fp64": g(line["value"]), "mixed": g(line["mixed"]["value"]),
                        "mixed_df": g(line["mixed_df"]["value"])},
           "quadrant_e2e": {"fp64": g(line["e2e"]["value"]),
                            "mixed": g(line["mixed"]["e2e"]["value"]),
                            "mixed_df": g(line["mixed_df"]["e2e"]["value"])},
           "fp64_hbm_frac": round(line["roofline"]["frac"], 4),
           "fp64_pipe_frac": round((line["roofline"].get("fp64_pipe") or {}).get("frac", 0.0), 4)}
    if line.get("cpu_baseline"):
        out["cpu_oracle"] = g(line["cpu_baseline"]["value"])
    kh = line.get("kelvin_helmholtz")
    if kh:
        out["kh"] = {p: g(kh[p]["value"]) for p in ("fp64", "mixed", "mixed_df") if p in kh}
    sl = line.get("slabs")
    if sl:
        out["slabs_2_on_1_gpu"] = {p: g(sl[p]["value"]) for p in ("fp64", "mixed") if p in sl}
    b = line.get("batched")
    if b:
        bt = {}
        for p in ("fp64", "mixed_df", "mixed"):
            if isinstance(b.get(p), dict) and "value" in b[p]:
                e = b[p].get("density_error_vs_fp64")
                bt[p] = {"value": g(b[p]["value"])}
                if e:
                    bt[p].update({"l1_median": e["rel_l1"]["median"], "l1_max": e["rel_l1"]["max"],
                                  "l1_above_1e-6": e["rel_l1"]["above_1e-6"],
                                  "instances": e["instances_compared"]})
        out["batched"] = bt
    sv = line.get("serving")
    if sv:
        out["serving_100_per_s"] = {
            p: {"completed": r["completed"], "p50_s": round(r["p50_latency_s"], 2),
                "p99_s": round(r["p99_latency_s"], 2), "value": g(r["cell_updates_per_s"])}
            for p, rows in sv.items() if isinstance(rows, list)
            for r in rows if r.get("rate_per_s") == 100.0}
    return out


if __name__ == "__main__":
    sys.exit(main())
