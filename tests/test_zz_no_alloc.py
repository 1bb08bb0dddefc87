"""cato_gpu_solve_noalloc: the residual entry point for callers that cannot allocate device
memory (their GPU memory belongs to another allocator, or an allocation would synchronize a
latency-critical loop).  It must give exactly what the allocating entry point cato_gpu_solve
gives (FP64: bit-identical), call after call, although every call reuses one fixed device array
that keeps the previous call's contents.

This file is collected last so that a run stopping at the first failure has run every other
test; it also passes on its own in a fresh process."""
import ctypes
import gc

import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300 import _lib
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import FluxSolver

pytestmark = pytest.mark.gpu

CATO_ERR_CAPACITY = 16


def _noalloc(L, cfg, prims):
    fn = L.cato_gpu_solve_noalloc
    dp = ctypes.POINTER(ctypes.c_double)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(type(cfg.to_c()))] + [dp] * 8 + [ctypes.c_int64]
    c = cfg.to_c()
    outs = [np.zeros(cfg.halo_shape, order="F") for _ in range(4)]
    rc = fn(ctypes.byref(c), *(_lib.ptr(a) for a in prims), *(_lib.ptr(a) for a in outs),
            cfg.halo_shape[0])
    return rc, outs


def _case(flux, limiter, bc, ni, nj, seed):
    cfg = SchemeConfig(ni=ni, nj=nj, dx=1.0 / ni, dy=0.5 / nj, flux_solver=flux, limiter=limiter,
                       bc=bc, gamma=1.4, cfl=0.4)
    return cfg, random_prims(cfg, np.random.default_rng(seed))


def test_noalloc_matches_allocating_entry_on_consecutive_calls():
    L = _lib.load(build_if_missing=True)
    cases = [
        _case("SD-SLAU", "MLP5", {"+x": "periodic", "-x": "periodic", "+y": "symmetry",
                                  "-y": "symmetry"}, 150, 47, 11),
        _case("Roe", "superbee", {"+x": "zero_gradient", "-x": "zero_gradient",
                                  "+y": "zero_gradient", "-y": "zero_gradient"}, 97, 61, 12),
    ]
    for cfg, prims in cases:  # two calls in a row, different sizes and schemes
        ref_in = [a.copy(order="F") for a in prims]
        ref = FluxSolver(cfg).solve(*ref_in)
        got_in = [a.copy(order="F") for a in prims]
        rc, got = _noalloc(L, cfg, got_in)
        assert rc == 0, rc
        for k in range(4):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"residual {k}")
            np.testing.assert_array_equal(got_in[k], ref_in[k], err_msg=f"ghosts {k}")


def test_noalloc_refuses_grids_beyond_its_capacity():
    L = _lib.load(build_if_missing=True)
    cfg, prims = _case("AUSMPW+", "minmod", {s: "zero_gradient" for s in ("+x", "-x", "+y", "-y")},
                       700, 700, 0)
    rc, _ = _noalloc(L, cfg, prims)
    assert rc == CATO_ERR_CAPACITY
    # the refusal leaves the shared array usable: a grid that fits still gives the residual
    cfg, prims = _case("AUSMPW+", "minmod", {s: "zero_gradient" for s in ("+x", "-x", "+y", "-y")},
                       64, 40, 1)
    ref = FluxSolver(cfg).solve(*[a.copy(order="F") for a in prims])
    rc, got = _noalloc(L, cfg, [a.copy(order="F") for a in prims])
    assert rc == 0, rc
    for k in range(4):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=f"residual {k}")


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found: cannot read the device's free memory")


def _free_bytes(rt):
    free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_takes_no_device_memory():
    """The device's free memory is the same before and after further calls of other sizes
    (each scheme runs once first, so that its kernels are loaded before the measurement)."""
    L = _lib.load(build_if_missing=True)
    rt = _cudart()
    zg = {s: "zero_gradient" for s in ("+x", "-x", "+y", "-y")}
    cases = [_case("HLLC", "van_leer", zg, 96, 80, 3), _case("HLLC", "van_leer", zg, 512, 500, 4),
             _case("HLLC", "van_leer", zg, 33, 17, 5)]
    rc, _ = _noalloc(L, cases[0][0], [a.copy(order="F") for a in cases[0][1]])
    assert rc == 0, rc
    gc.collect()
    before = _free_bytes(rt)
    for _ in range(2):
        for cfg, prims in cases:
            rc, _ = _noalloc(L, cfg, [a.copy(order="F") for a in prims])
            assert rc == 0, rc
    assert _free_bytes(rt) == before
