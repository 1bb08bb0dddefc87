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
# algorithmic HBM bytes per cell and stage kernel launch (state in, state out), SSP-RK3:
#   FP64 : stage 1 reads U^n, writes U1 (64 B); stages 2, 3 read U^n + U^k, write 32 B (96 B)
#   mixed: stage 1 reads U^n, writes delta1 (32+16); stage 2 reads U^n + delta1, writes delta2
#          (32+16+16); stage 3 reads U^n + delta2, writes U^{n+1} (32+16+32)
BYTES_PER_CELL_STAGE = {"fp64": (64, 96, 96), "mixed": (48, 64, 80)}


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
        "config": workload_config(args, world),
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
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def bench_precision(args, precision, dist, world, peak_gbs):
    from fvleg_2d_gb300 import ic
    from fvleg_2d_gb300.fluid import Fluid

    cfg, prims = ic.riemann_quadrant(args.n, precision=precision)
    f = Fluid(cfg).initialize(*prims)
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
    }
    f.close()
    return res, cfg, prims


def bench_e2e(args, cfg, prims):
    """Through the C-ABI with pinned host buffers: upload, per-step integrate (dt and error code
    back to the host each step), download of the final conserved state."""
    import ctypes

    from fvleg_2d_gb300 import _lib
    from fvleg_2d_gb300.fluid import Fluid

    pinned = [_lib.PinnedArray(cfg.halo_shape) for _ in range(8)]
    for k in range(4):
        pinned[k].array[...] = prims[k]
    f = Fluid(cfg)
    # warm-up on the same handle (allocations, module load)
    f.initialize(*(p.array for p in pinned[:4]))
    for _ in range(min(args.warmup, 2)):
        f.integrate()
    L, h, ld = f.L, f.h, f.ld
    used, ec = ctypes.c_double(), ctypes.c_int32()
    t0 = time.perf_counter()
    rc = L.cato_gpu_upload_primitive(h, *(_lib.ptr(p.array) for p in pinned[:4]), ld)
    for _ in range(args.steps):
        rc |= L.cato_gpu_integrate(h, 0.0, ctypes.byref(used), ctypes.byref(ec))
    rc |= L.cato_gpu_download(h, *(_lib.ptr(p.array) for p in pinned[4:8]), None, None, None,
                              None, ld)
    secs = time.perf_counter() - t0
    if rc or ec.value:
        raise RuntimeError(f"e2e run failed rc={rc} ec={ec.value}")
    f.close()
    for p in pinned:
        p.free()
    cells = cfg.ni * cfg.nj
    state_bytes = 4 * cells * 8
    ctl = 72  # step-control block each way per integrate call
    return {"value": cells * args.steps / secs, "unit": "cell-updates/s",
            "h2d_bytes_per_step": state_bytes / args.steps + ctl,
            "d2h_bytes_per_step": state_bytes / args.steps + 2 * ctl,
            "sequence": "upload_primitive + K x integrate + download (pinned host buffers)"}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--cpu-baseline-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank, dist)

    from fvleg_2d_gb300 import _lib

    _lib.load(build_if_missing=True).cato_gpu_select_device(local)
    peak, peak_kind = measured_peaks()
    fp64, cfg, prims = bench_precision(args, "fp64", dist, world, peak)
    mixed, _, _ = bench_precision(args, "mixed", dist, world, peak)
    e2e = bench_e2e(args, cfg, prims)
    e2e_all = allreduce_max(dist, -e2e["value"])  # slowest replica
    e2e["value"] = -e2e_all * world
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, used, secs = cpu_reference(cfg, prims, args.cpu_baseline_steps, 0, threads)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": used, "kind": "port",
               "sample": f"{args.cpu_baseline_steps} SSP-RK3 steps of the same {args.n}^2 grid "
                         f"({secs:.1f} s, OpenMP C restatement of the reference)"}
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
        "config": workload_config(args, world),
        "hbm_gbs": fp64["roofline"]["achieved"],
        "roofline": dict(fp64["roofline"], peak_source=f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                         if peak_kind == "measured" else "fallback 6.8 TB/s"),
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": fp64["clocks"],
        "stage_ms_per_step": fp64["stage_ms_per_step"],
        "mixed": {
            "value": mixed["value"], "unit": "cell-updates/s", "dtype": "f32 flux / f64 state",
            "ms_per_step": mixed["ms_per_step"], "speedup_vs_fp64": mixed["value"] / fp64["value"],
            "roofline": mixed["roofline"], "stage_ms_per_step": mixed["stage_ms_per_step"],
            "gpu_launches": mixed["launches_per_step"] * args.steps, "clocks": mixed["clocks"],
        },
    }
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
