"""ctypes binding of ``libcato_gpu.so`` (the C-ABI of ``include/cato_gpu.h``).

The library is built in-tree by ``fvleg_2d_gb300.build``; there is no CPU fallback: if the
library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from .config import CatoConfig

_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


class CatoLibraryError(RuntimeError):
    pass


def lib_path() -> str:
    from . import build

    return build.lib_path()


def load(build_if_missing: bool = False):
    """Load libcato_gpu.so; with build_if_missing compile it first when absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise CatoLibraryError(
                f"{path} is missing: build it with `python -m fvleg_2d_gb300.build`")
        from . import build

        build.build()
    try:
        L = ctypes.CDLL(path)
    except OSError as exc:
        raise CatoLibraryError(f"cannot load {path}: {exc}") from exc
    H = ctypes.c_void_p
    cfgp = ctypes.POINTER(CatoConfig)
    i64 = ctypes.c_int64
    sig = {
        "cato_gpu_version": (ctypes.c_char_p, []),
        "cato_config_default": (ctypes.c_int, [cfgp, ctypes.c_int32, ctypes.c_int32]),
        "cato_config_check": (ctypes.c_int, [cfgp]),
        "cato_gpu_create": (ctypes.c_int, [cfgp, ctypes.POINTER(H)]),
        "cato_gpu_destroy": (ctypes.c_int, [H]),
        "cato_gpu_last_error": (ctypes.c_char_p, [H]),
        "cato_gpu_upload_primitive": (ctypes.c_int, [H, _dp, _dp, _dp, _dp, i64]),
        "cato_gpu_set_rectilinear": (ctypes.c_int, [H, _dp, _dp]),
        "cato_gpu_set_bc_table": (ctypes.c_int, [H, ctypes.c_int32, _dp, _dp, _dp]),
        "cato_gpu_set_energy_source": (ctypes.c_int, [H, ctypes.c_void_p, ctypes.c_int32,
                                                      _dp, _dp, _dp]),
        "cato_gpu_get_timestep": (ctypes.c_int, [H, _dp]),
        "cato_gpu_integrate": (ctypes.c_int, [H, ctypes.c_double, _dp,
                                              ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_run": (ctypes.c_int, [H, i64, ctypes.c_double, ctypes.POINTER(i64), _dp,
                                        ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_set_time": (ctypes.c_int, [H, ctypes.c_double, i64]),
        "cato_gpu_get_time": (ctypes.c_int, [H, _dp, ctypes.POINTER(i64), _dp]),
        "cato_gpu_download": (ctypes.c_int, [H] + [_dp] * 8 + [i64]),
        "cato_gpu_conservation_sums": (ctypes.c_int, [H, _dp]),
        "cato_gpu_convergence": (ctypes.c_int, [H, _dp]),
        "cato_gpu_set_step_options": (ctypes.c_int, [H, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.c_double]),
        "cato_gpu_step_begin": (ctypes.c_int, [H, ctypes.c_double]),
        "cato_gpu_step_stage": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_step_end": (ctypes.c_int, [H, _dp, ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_halo_export": (ctypes.c_int, [H, ctypes.c_int32, _dp]),
        "cato_gpu_halo_import": (ctypes.c_int, [H, ctypes.c_int32, _dp]),
        "cato_gpu_solve": (ctypes.c_int, [H] + [_dp] * 8 + [i64]),
        "cato_gpu_interpolate_edges": (ctypes.c_int, [H, _dp, i64, _dp, _dp]),
        "cato_gpu_status": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_synchronize": (ctypes.c_int, [H]),
        "cato_gpu_set_stream": (ctypes.c_int, [H, ctypes.c_void_p]),
        "cato_gpu_profile_step": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_float), ctypes.c_int32,
                                                 ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_launches_per_step": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_run_timed": (ctypes.c_int, [H, i64, ctypes.POINTER(ctypes.c_float),
                                              ctypes.POINTER(ctypes.c_float), ctypes.c_int32]),
        "cato_gpu_select_device": (ctypes.c_int, [ctypes.c_int32]),
        "cato_gpu_set_kernel_variant": (ctypes.c_int, [H, ctypes.c_int32]),
        "cato_gpu_get_kernel_variant": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_tune": (ctypes.c_int, [H, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_float)]),
        "cato_gpu_check_divsqrt": (ctypes.c_int, [ctypes.c_int64, ctypes.c_uint64,
                                                  ctypes.POINTER(ctypes.c_uint64),
                                                  ctypes.POINTER(ctypes.c_uint64),
                                                  ctypes.POINTER(ctypes.c_int32)]),
        "cato_gpu_set_plan": (ctypes.c_int, [H, ctypes.c_int32, ctypes.c_int32]),
        "cato_gpu_get_plan": (ctypes.c_int, [H, ctypes.POINTER(ctypes.c_int32),
                                             ctypes.POINTER(ctypes.c_int32)]),
        "cato_host_alloc": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
        "cato_host_free": (ctypes.c_int, [ctypes.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return _lib


class PinnedArray:
    """A Fortran-ordered float64 numpy view of page-locked host memory (cato_host_alloc)."""

    def __init__(self, shape):
        import numpy as np

        n = int(np.prod(shape)) * 8
        self._p = ctypes.c_void_p()
        rc = load().cato_host_alloc(n, ctypes.byref(self._p))
        if rc != 0:
            raise CatoLibraryError(f"cato_host_alloc({n}) failed: {rc}")
        buf = (ctypes.c_double * (n // 8)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(shape, order="F")

    def free(self):
        if self._p:
            self.array = None
            load().cato_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def ptr(a) -> "ctypes._Pointer":
    if a is None:
        return None
    assert a.dtype.itemsize == 8 and a.flags.f_contiguous, "float64 Fortran-ordered array expected"
    return a.ctypes.data_as(_dp)
