"""Batched engine: many independent grid instances of uneven sizes advanced together on one GPU
(``cato_batch_*`` in ``include/cato_gpu.h``).

Each instance has its own state, CFL dt, time, iteration count and stop condition; a step of the
batch is one persistent launch per RK stage (per flux/reconstruction group) whose CTAs pull
(instance, tile) work items from a device queue, and chunks of steps replay a captured CUDA
graph.  An instance's results do not depend on the other instances in the batch.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .config import PRECISION_IDS, RK_IDS, CatoConfig, SchemeConfig
from .fluid import CatoError, _check


def _sig(L):
    if getattr(L, "_batch_sig", False):
        return
    B = ctypes.c_void_p
    cfgp = ctypes.POINTER(CatoConfig)
    dp = ctypes.POINTER(ctypes.c_double)
    i32p = ctypes.POINTER(ctypes.c_int32)
    sig = {
        "cato_batch_create": [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(B)],
        "cato_batch_destroy": [B],
        "cato_batch_instance_bytes": [cfgp, ctypes.POINTER(ctypes.c_uint64)],
        "cato_batch_add": [B, cfgp, dp, dp, dp, dp, ctypes.c_int64, ctypes.c_double,
                           ctypes.c_int64, i32p],
        "cato_batch_remove": [B, ctypes.c_int32],
        "cato_batch_set_plan": [B, ctypes.c_int32, ctypes.c_int32],
        "cato_batch_step": [B, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)],
        "cato_batch_query": [B, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64), dp, dp, i32p, i32p],
        "cato_batch_running": [B, i32p, i32p],
        "cato_batch_download": [B, ctypes.c_int32, dp, dp, dp, dp, ctypes.c_int64],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    L._batch_sig = True


def instance_bytes(cfg: SchemeConfig) -> int:
    L = _lib.load()
    _sig(L)
    n = ctypes.c_uint64()
    c = cfg.to_c()
    _check(L.cato_batch_instance_bytes(ctypes.byref(c), ctypes.byref(n)))
    return n.value


class Batch:
    def __init__(self, capacity: int, precision: str = "mixed", integration_strategy: str = "ssp_rk2"):
        self.L = _lib.load()
        _sig(self.L)
        self.capacity = capacity
        self.precision = precision
        self.rk = integration_strategy
        h = ctypes.c_void_p()
        _check(self.L.cato_batch_create(capacity, PRECISION_IDS[precision], RK_IDS[integration_strategy],
                                        ctypes.byref(h)), None, "cato_batch_create")
        self.h = h
        self.cfgs: dict[int, SchemeConfig] = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.cato_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, cfg: SchemeConfig, prims, t_end: float = float("inf"), max_steps: int = -1) -> int:
        if cfg.precision != self.precision or cfg.integration_strategy != self.rk:
            raise ValueError("instance precision / integrator differ from the batch's")
        c = cfg.to_c()
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in prims]
        slot = ctypes.c_int32()
        _check(self.L.cato_batch_add(self.h, ctypes.byref(c), *(_lib.ptr(a) for a in arrs),
                                     cfg.halo_shape[0], float(t_end), int(max_steps),
                                     ctypes.byref(slot)), None, "cato_batch_add")
        self.cfgs[slot.value] = cfg
        return slot.value

    def remove(self, slot: int) -> None:
        _check(self.L.cato_batch_remove(self.h, int(slot)), None, "cato_batch_remove")
        self.cfgs.pop(slot, None)

    def set_plan(self, threads: int, rows_per_cta: int) -> None:
        _check(self.L.cato_batch_set_plan(self.h, int(threads), int(rows_per_cta)))

    def step(self, n_steps: int, use_graph: bool = True) -> float:
        """Advance n_steps; returns the device time in ms."""
        ms = ctypes.c_float()
        _check(self.L.cato_batch_step(self.h, int(n_steps), 1 if use_graph else 0,
                                      ctypes.byref(ms)), None, "cato_batch_step")
        return ms.value

    def query(self, slot: int) -> dict:
        it, t, dt = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        run, ec = ctypes.c_int32(), ctypes.c_int32()
        _check(self.L.cato_batch_query(self.h, int(slot), ctypes.byref(it), ctypes.byref(t),
                                       ctypes.byref(dt), ctypes.byref(run), ctypes.byref(ec)))
        return {"iteration": it.value, "time": t.value, "dt": dt.value, "running": bool(run.value),
                "error_code": ec.value}

    def running(self):
        n = ctypes.c_int32()
        flags = (ctypes.c_int32 * self.capacity)()
        _check(self.L.cato_batch_running(self.h, ctypes.byref(n), flags))
        return n.value, [bool(f) for f in flags]

    def state(self, slot: int) -> dict:
        cfg = self.cfgs[slot]
        out = {k: np.zeros(cfg.halo_shape, order="F") for k in ("rho", "rho_u", "rho_v", "rho_E")}
        _check(self.L.cato_batch_download(self.h, int(slot), *(_lib.ptr(out[k]) for k in
                                          ("rho", "rho_u", "rho_v", "rho_E")), cfg.halo_shape[0]))
        return out

    def run_until_done(self, chunk: int = 64, max_chunks: int = 10**6) -> tuple[int, float]:
        """Step until no instance is running; returns (steps issued, device ms)."""
        total_ms, steps = 0.0, 0
        for _ in range(max_chunks):
            n, _flags = self.running()
            if n == 0:
                break
            total_ms += self.step(chunk)
            steps += chunk
        return steps, total_ms


__all__ = ["Batch", "instance_bytes", "CatoError"]
