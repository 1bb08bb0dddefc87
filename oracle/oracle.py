"""TEST INFRASTRUCTURE ONLY: Python binding of the C parity oracle (``oracle/cato_oracle.c``).

The oracle restates the reference's FP64 arithmetic on the CPU.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this module; the product
package ``fvleg_2d_gb300`` never does.

Fields are numpy float64 arrays of shape ``(ni + 2*ng, nj + 2*ng)`` in Fortran order, i.e. the
reference's ``field_2d_t%data`` with bounds ``(1-ng:ni+ng, 1-ng:nj+ng)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from fvleg_2d_gb300.config import CatoConfig, SchemeConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcato_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
# oracle_exchange_fn(user, rho, u, v, p)
_XCHG = ctypes.CFUNCTYPE(None, ctypes.c_void_p, _dp, _dp, _dp, _dp)


def build() -> str:
    """Compile the oracle (make in oracle/); returns the library path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        cfgp = ctypes.POINTER(CatoConfig)
        L.oracle_set_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_get_threads.restype = ctypes.c_int
        L.oracle_config_check.argtypes = [cfgp]
        L.oracle_limiter.restype = ctypes.c_double
        L.oracle_limiter.argtypes = [ctypes.c_int32, ctypes.c_double]
        L.oracle_quad_metrics.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_apply_bc.argtypes = [cfgp, _dp, _dp, _dp, _dp]
        L.oracle_apply_bc_side.argtypes = [cfgp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           _dp, _dp, _dp, _dp]
        L.oracle_interpolate_edges.argtypes = [cfgp, _dp, _dp, _dp]
        L.oracle_solve.argtypes = [cfgp] + [_dp] * 8
        L.oracle_solve_rect.argtypes = [cfgp] + [_dp] * 10
        L.oracle_set_rectilinear.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.oracle_set_time.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int64]
        L.oracle_set_subcycle.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.oracle_set_exchange.argtypes = [ctypes.c_void_p, _XCHG, ctypes.c_void_p]
        L.oracle_dt.restype = ctypes.c_double
        L.oracle_dt.argtypes = [ctypes.c_void_p]
        L.oracle_set_pow_mode.argtypes = [ctypes.c_int]
        L.oracle_set_energy_source.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                               _dp, _dp, _dp]
        L.oracle_source_field.argtypes = [ctypes.c_void_p, _dp]
        L.oracle_pow.restype = ctypes.c_double
        L.oracle_pow.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oracle_set_bc_table.argtypes = [ctypes.c_void_p, ctypes.c_int32, _dp, _dp, _dp]
        L.oracle_solve_pbc.argtypes = ([cfgp, ctypes.c_int32, _dp, _dp, _dp, ctypes.c_double]
                                       + [_dp] * 8)
        L.oracle_create.restype = ctypes.c_void_p
        L.oracle_create.argtypes = [cfgp]
        L.oracle_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_set_primitive.restype = ctypes.c_int
        L.oracle_set_primitive.argtypes = [ctypes.c_void_p] + [_dp] * 4
        L.oracle_set_conserved.argtypes = [ctypes.c_void_p] + [_dp] * 4
        L.oracle_get_timestep.restype = ctypes.c_double
        L.oracle_get_timestep.argtypes = [ctypes.c_void_p]
        L.oracle_integrate.argtypes = [ctypes.c_void_p, ctypes.c_double,
                                       ctypes.POINTER(ctypes.c_int32)]
        L.oracle_get_state.argtypes = [ctypes.c_void_p] + [_dp] * 8
        L.oracle_time.restype = ctypes.c_double
        L.oracle_time.argtypes = [ctypes.c_void_p]
        L.oracle_iteration.restype = ctypes.c_int64
        L.oracle_iteration.argtypes = [ctypes.c_void_p]
        for name in ("oracle_convergence", "oracle_conservation_sums"):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.f_contiguous
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


def limiter(name_or_id, r: float) -> float:
    from fvleg_2d_gb300.config import LIMITER_IDS

    lid = LIMITER_IDS[name_or_id] if isinstance(name_or_id, str) else int(name_or_id)
    return lib().oracle_limiter(lid, float(r))


def quad_metrics(x, y):
    """quad_cell_t metrics of a cell with nodes (x[k], y[k]), k = 1..4 counter-clockwise."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    vol = np.zeros(1)
    el = np.zeros(4)
    nv = np.zeros(8)
    mdx = np.zeros(1)
    mdy = np.zeros(1)
    lib().oracle_quad_metrics(*(a.ctypes.data_as(_dp) for a in (x, y, vol, el, nv, mdx, mdy)))
    return {"volume": vol[0], "edge_lengths": el, "edge_norm_vectors": nv.reshape(4, 2),
            "min_dx": mdx[0], "min_dy": mdy[0]}


def _cfg(cfg):
    return ctypes.byref(cfg.to_c() if isinstance(cfg, SchemeConfig) else cfg)


def empty_field(cfg: SchemeConfig) -> np.ndarray:
    return np.zeros(cfg.halo_shape, dtype=np.float64, order="F")


def apply_bc(cfg: SchemeConfig, rho, u, v, p) -> None:
    """In place, like flux_solver_t%apply_primitive_bc."""
    lib().oracle_apply_bc(_cfg(cfg), _ptr(rho), _ptr(u), _ptr(v), _ptr(p))


def apply_bc_side(cfg: SchemeConfig, side: str, bc_type: str, do_corners: bool, rho, u, v, p):
    """One boundary condition on one side ('+x', '+y', '-x', '-y'), in place."""
    from fvleg_2d_gb300.config import BC_IDS, SIDES

    lib().oracle_apply_bc_side(_cfg(cfg), SIDES.index(side), BC_IDS[bc_type], int(do_corners),
                               _ptr(rho), _ptr(u), _ptr(v), _ptr(p))


def interpolate_edges(cfg: SchemeConfig, q):
    """Returns (i_edges(2, -1:ni, 0:nj), j_edges(2, 0:ni, -1:nj)) as Fortran-order arrays."""
    ni, nj = cfg.ni, cfg.nj
    ie = np.zeros((2, ni + 2, nj + 1), order="F")
    je = np.zeros((2, ni + 1, nj + 2), order="F")
    lib().oracle_interpolate_edges(_cfg(cfg), _ptr(q), _ptr(ie), _ptr(je))
    return ie, je


class pow_mode:
    """Context: the pressure-input inlet's powers in the oracle, "libm" (the reference's pow)
    or "cr" (correctly rounded, the arithmetic of the CUDA path)."""

    def __init__(self, mode: str):
        self.mode = {"libm": 0, "cr": 1}[mode]

    def __enter__(self):
        lib().oracle_set_pow_mode(self.mode)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_pow_mode(0)


def solve(cfg: SchemeConfig, rho, u, v, p, nodes=None, bc_table=None, time=0.0):
    """flux_solver_t%solve: BCs written into the ghosts of rho/u/v/p; returns d/dt of U.
    ``nodes = (x(1..ni+1), y(1..nj+1))`` selects a rectilinear grid; ``bc_table = (t, p, rho)``
    a tabulated pressure-input target evaluated at ``time``."""
    out = [empty_field(cfg) for _ in range(4)]
    if bc_table is not None:
        t, pt, rt = (np.ascontiguousarray(a, dtype=np.float64) for a in bc_table)
        rc = lib().oracle_solve_pbc(_cfg(cfg), len(t), t.ctypes.data_as(_dp),
                                    pt.ctypes.data_as(_dp), rt.ctypes.data_as(_dp), float(time),
                                    _ptr(rho), _ptr(u), _ptr(v), _ptr(p), *(_ptr(a) for a in out))
    elif nodes is None:
        rc = lib().oracle_solve(_cfg(cfg), _ptr(rho), _ptr(u), _ptr(v), _ptr(p),
                                *(_ptr(a) for a in out))
    else:
        xs, ys = (np.ascontiguousarray(a, dtype=np.float64) for a in nodes)
        rc = lib().oracle_solve_rect(_cfg(cfg), xs.ctypes.data_as(_dp), ys.ctypes.data_as(_dp),
                                     _ptr(rho), _ptr(u), _ptr(v), _ptr(p),
                                     *(_ptr(a) for a in out))
    if rc != 0:
        raise RuntimeError(f"oracle_solve failed: {rc}")
    return out


class OracleFluid:
    """fluid_t restated on the CPU."""

    def __init__(self, cfg: SchemeConfig):
        self.cfg = cfg
        self._c = cfg.to_c()
        self._h = lib().oracle_create(ctypes.byref(self._c))
        if not self._h:
            raise ValueError("invalid configuration")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_destroy(h)
            self._h = None

    def set_rectilinear(self, x_nodes, y_nodes) -> None:
        """Rectilinear grid of node coordinates x(1..ni+1), y(1..nj+1)."""
        xs, ys = (np.ascontiguousarray(a, dtype=np.float64) for a in (x_nodes, y_nodes))
        rc = lib().oracle_set_rectilinear(self._h, xs.ctypes.data_as(_dp),
                                          ys.ctypes.data_as(_dp))
        if rc:
            raise ValueError(f"oracle_set_rectilinear: {rc}")

    def set_time(self, time: float, iteration: int) -> None:
        lib().oracle_set_time(self._h, float(time), int(iteration))

    def set_subcycle(self, allow: bool, tolerance: float = 1e-3) -> None:
        """[time] allow_subcycle / subcycle_error_tolerance: SSP steps repeat with dt / 10
        while a convergence norm exceeds the tolerance."""
        lib().oracle_set_subcycle(self._h, int(bool(allow)), float(tolerance))

    @property
    def dt(self) -> float:
        """dt of the last step (after any subcycling)."""
        return lib().oracle_dt(self._h)

    def set_exchange(self, fn) -> None:
        """Slab of a row-split grid: ``fn(q)`` gets the four halo-padded primitive fields
        (rho, u, v, p; views, Fortran order) of every residual evaluation before the boundary
        conditions and writes the ghost rows beyond the exchange sides.  None removes it."""
        if fn is None:
            self._xchg = None
            lib().oracle_set_exchange(self._h, _XCHG(), None)
            return
        shape = self.cfg.halo_shape
        n = shape[0] * shape[1]

        def cb(_user, r, u, v, p):
            fn([np.ctypeslib.as_array(a, shape=(n,)).reshape(shape, order="F")
                for a in (r, u, v, p)])

        self._xchg = _XCHG(cb)  # kept alive while the oracle may call it
        lib().oracle_set_exchange(self._h, self._xchg, None)

    def set_energy_source(self, source=None) -> None:
        """An EnergySource (fvleg_2d_gb300.config) or None."""
        if source is None:
            lib().oracle_set_energy_source(self._h, None, 0, None, None, None)
            return
        self._src_c = source.to_c()
        if source.table is None:
            self._src_tab, n, ptrs = None, 0, [None] * 3
        else:
            self._src_tab = [np.ascontiguousarray(a, dtype=np.float64) for a in source.table]
            n = len(self._src_tab[0])
            ptrs = [a.ctypes.data_as(_dp) for a in self._src_tab]
        rc = lib().oracle_set_energy_source(self._h, ctypes.byref(self._src_c), n, *ptrs)
        if rc:
            raise ValueError(f"oracle_set_energy_source: {rc}")

    def set_bc_table(self, time, pressure, density) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (time, pressure, density)]
        rc = lib().oracle_set_bc_table(self._h, len(arrs[0]),
                                       *(a.ctypes.data_as(_dp) for a in arrs))
        if rc:
            raise ValueError(f"oracle_set_bc_table: {rc}")

    def source_field(self) -> np.ndarray:
        """q_dot_h for a step starting now, (ni, nj)."""
        out = np.zeros((self.cfg.ni, self.cfg.nj), order="F")
        rc = lib().oracle_source_field(self._h, _ptr(out))
        if rc:
            raise RuntimeError(f"oracle_source_field: {rc}")
        return out

    def set_primitive(self, rho, u, v, p) -> int:
        """Load a primitive state; returns initialize_from_hdf5's verdict on it (0, or
        NEG_PRESSURE / NEG_DENSITY for a pressure / density below tiny)."""
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in (rho, u, v, p)]
        return lib().oracle_set_primitive(self._h, *(_ptr(a) for a in arrs))

    def set_conserved(self, rho, rho_u, rho_v, rho_E) -> None:
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in (rho, rho_u, rho_v, rho_E)]
        lib().oracle_set_conserved(self._h, *(_ptr(a) for a in arrs))

    def get_timestep(self) -> float:
        return lib().oracle_get_timestep(self._h)

    def integrate(self, dt: float | None = None) -> int:
        if dt is None or dt <= 0:
            dt = self.get_timestep()
        ec = ctypes.c_int32(0)
        rc = lib().oracle_integrate(self._h, float(dt), ctypes.byref(ec))
        if rc != 0:
            raise RuntimeError(f"oracle_integrate failed: {rc}")
        self.last_dt = dt
        return ec.value

    def state(self) -> dict:
        names = ("rho", "rho_u", "rho_v", "rho_E", "u", "v", "p", "cs")
        out = {k: empty_field(self.cfg) for k in names}
        lib().oracle_get_state(self._h, *(_ptr(out[k]) for k in names))
        return out

    @property
    def time(self) -> float:
        return lib().oracle_time(self._h)

    @property
    def iteration(self) -> int:
        return lib().oracle_iteration(self._h)

    def convergence(self) -> np.ndarray:
        """calculate_convergence of the last step: [rho, rho u, rho v, rho E]."""
        out = np.zeros(4)
        rc = lib().oracle_convergence(self._h, _ptr(out))
        if rc:
            raise RuntimeError(f"oracle_convergence: {rc}")
        return out

    def conservation_sums(self) -> np.ndarray:
        """Interior totals of rho, rho u, rho v, rho E times the cell volume."""
        out = np.zeros(4)
        lib().oracle_conservation_sums(self._h, _ptr(out))
        return out

    def run(self, t_end: float, max_steps: int = 10**9) -> int:
        """The main.f90 time loop (CFL dt each step, no last-step trim); returns steps taken."""
        n = 0
        while self.time < t_end and n < max_steps:
            ec = self.integrate()
            n += 1
            if ec != 0:
                raise RuntimeError(f"fluid error code {ec} at step {n}")
        return n
