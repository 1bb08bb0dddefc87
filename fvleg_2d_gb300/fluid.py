"""Host-side mirror of the reference's interfaces for the time-step hot path.

* :class:`Fluid`          -- ``fluid_t`` (``src/lib/fluid/mod_fluid.f90:68-141``): ``integrate``,
  ``get_timestep``, ``set_time``, ``t`` (time derivative) and the conserved/derived fields.
* :class:`FluxSolver`     -- ``flux_solver_t%solve`` (``src/lib/flux_solvers/flux_solver.f90:66-87``).
* :class:`MusclInterpolator` -- ``muscl_interpolation_t%interpolate_edge_values``
  (``src/lib/spatial_reconstruction/muscl_interpolation.f90:37-43``).

All arithmetic runs on the GPU through ``libcato_gpu.so``; these classes only move arrays across
the C-ABI.  Where the reference stops the program (``error stop``), these raise
:class:`CatoError` carrying the reference's error code.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .config import SIDES, STATUS_NAMES, SchemeConfig


class CatoError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        self.code = code
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}".rstrip(": "))


def _check(rc: int, h=None, what: str = ""):
    if rc != 0:
        msg = ""
        if h is not None:
            m = _lib.load().cato_gpu_last_error(h)
            msg = m.decode() if m else ""
        raise CatoError(rc, f"{what} {msg}".strip())


def _c_ptr(a: np.ndarray):
    """Pointer to a C-contiguous float64 array (the slab edge rows)."""
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _field(cfg: SchemeConfig) -> np.ndarray:
    return np.zeros(cfg.halo_shape, dtype=np.float64, order="F")


def _as_field(cfg: SchemeConfig, a) -> np.ndarray:
    a = np.asfortranarray(a, dtype=np.float64)
    if a.shape != cfg.halo_shape:
        raise ValueError(f"field shape {a.shape} != halo-padded shape {cfg.halo_shape}")
    return a


class _Handle:
    def __init__(self, cfg: SchemeConfig):
        self.cfg = cfg
        self.L = _lib.load()
        self._c = cfg.to_c()
        h = ctypes.c_void_p()
        _check(self.L.cato_gpu_create(ctypes.byref(self._c), ctypes.byref(h)), None,
               "cato_gpu_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.cato_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ld(self) -> int:
        return self.cfg.halo_shape[0]

    def set_rectilinear(self, x_nodes, y_nodes):
        """Non-uniform tensor-product grid: interior node coordinates x(1..ni+1), y(1..nj+1),
        strictly increasing (the uniform and layered grids of pycato's
        generate_initial_grids.py:43-380, whose cells are axis-aligned).  ``None, None`` returns
        to the configuration's uniform dx x dy.  Call before ``initialize``."""
        if x_nodes is None and y_nodes is None:
            xs = ys = None
        else:
            xs = np.ascontiguousarray(x_nodes, dtype=np.float64)
            ys = np.ascontiguousarray(y_nodes, dtype=np.float64)
            if xs.shape != (self.cfg.ni + 1,) or ys.shape != (self.cfg.nj + 1,):
                raise ValueError(f"expected {self.cfg.ni + 1} x nodes and {self.cfg.nj + 1} "
                                 f"y nodes, got {xs.shape} and {ys.shape}")
        _check(self.L.cato_gpu_set_rectilinear(self.h, _lib.ptr(xs), _lib.ptr(ys)), self.h,
               "set_rectilinear")
        self.nodes = None if xs is None else (xs, ys)
        return self

    def set_bc_table(self, time=None, pressure=None, density=None):
        """Target of the +x 'pressure_input' side as a table in time (non-dimensional time,
        pressure and density as read_pressure_input leaves them, pressure_input_bc.f90:92-181);
        no arguments returns to the configuration's constant target."""
        if time is None:
            _check(self.L.cato_gpu_set_bc_table(self.h, 0, None, None, None), self.h,
                   "set_bc_table")
            self.bc_table = None
            return self
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (time, pressure, density)]
        n = arrs[0].shape[0]
        if any(a.shape != (n,) for a in arrs):
            raise ValueError("time, pressure and density must be 1-D arrays of one length")
        _check(self.L.cato_gpu_set_bc_table(self.h, n, *(_lib.ptr(a) for a in arrs)), self.h,
               "set_bc_table")
        self.bc_table = tuple(arrs)
        return self

    def set_energy_source(self, source=None):
        """The energy source term (an EnergySource; None turns it off).  Its field is
        recomputed at every step start and added to the energy equation at every stage."""
        if source is None:
            _check(self.L.cato_gpu_set_energy_source(self.h, None, 0, None, None, None), self.h,
                   "set_energy_source")
            self.source = None
            return self
        c = source.to_c()
        if source.table is None:
            arrs, n = [None] * 3, 0
        else:
            arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in source.table]
            n = arrs[0].shape[0]
            if any(a.shape != (n,) for a in arrs):
                raise ValueError("the source table needs three 1-D arrays of one length")
        _check(self.L.cato_gpu_set_energy_source(
            self.h, ctypes.byref(c), n, *(None if a is None else _lib.ptr(a) for a in arrs)),
            self.h, "set_energy_source")
        self.source = source
        return self

    def set_time(self, time: float, iteration: int) -> None:
        """fluid_t%set_time (mod_fluid.f90:400-409); also the time at which a FluxSolver
        evaluates a tabulated pressure-input target."""
        _check(self.L.cato_gpu_set_time(self.h, float(time), int(iteration)), self.h, "set_time")

    @property
    def time(self) -> float:
        t = ctypes.c_double()
        _check(self.L.cato_gpu_get_time(self.h, ctypes.byref(t), None, None), self.h)
        return t.value

    @property
    def iteration(self) -> int:
        it = ctypes.c_int64()
        _check(self.L.cato_gpu_get_time(self.h, None, ctypes.byref(it), None), self.h)
        return it.value

    @property
    def last_dt(self) -> float:
        """dt of the last step taken (0 before the first)."""
        dt = ctypes.c_double()
        _check(self.L.cato_gpu_get_time(self.h, None, None, ctypes.byref(dt)), self.h)
        return dt.value


class Fluid(_Handle):
    """fluid_t on the GPU.  ``Fluid(cfg).initialize(rho, u, v, p)`` replaces
    fluid_t%initialize + initialize_from_hdf5 (mod_fluid.f90:159-381)."""

    def initialize(self, rho, u, v, p) -> "Fluid":
        arrs = [_as_field(self.cfg, a) for a in (rho, u, v, p)]
        _check(self.L.cato_gpu_upload_primitive(self.h, *(_lib.ptr(a) for a in arrs), self.ld),
               self.h, "initialize")
        return self

    def get_timestep(self) -> float:
        dt = ctypes.c_double()
        _check(self.L.cato_gpu_get_timestep(self.h, ctypes.byref(dt)), self.h, "get_timestep")
        return dt.value

    def integrate(self, dt: float | None = None) -> tuple[float, int]:
        """One time step; dt=None uses the CFL dt (master_puppeteer.f90:166-170).
        Returns (dt taken, error_code)."""
        used = ctypes.c_double()
        ec = ctypes.c_int32()
        _check(self.L.cato_gpu_integrate(self.h, float(dt) if dt else 0.0, ctypes.byref(used),
                                         ctypes.byref(ec)), self.h, "integrate")
        return used.value, ec.value

    # stage-by-stage stepping of a slab (``exchange`` sides): see fvleg_2d_gb300.slabs
    def step_begin(self, dt: float | None = None) -> None:
        """Open a step with this dt (the slabs' minimum CFL dt); None: the own CFL dt."""
        _check(self.L.cato_gpu_step_begin(self.h, float(dt) if dt else 0.0), self.h, "step_begin")

    def step_stage(self) -> int:
        """Run the next RK stage of the open step; returns the stages still to run."""
        left = ctypes.c_int32()
        _check(self.L.cato_gpu_step_stage(self.h, ctypes.byref(left)), self.h, "step_stage")
        return left.value

    def step_end(self) -> tuple[float, int]:
        """Close the step: (dt taken, error code)."""
        used = ctypes.c_double()
        ec = ctypes.c_int32()
        _check(self.L.cato_gpu_step_end(self.h, ctypes.byref(used), ctypes.byref(ec)), self.h,
               "step_end")
        return used.value, ec.value

    def stage_count(self) -> int:
        n = ctypes.c_int32()
        _check(self.L.cato_gpu_launches_per_step(self.h, ctypes.byref(n)), self.h)
        return n.value - 1

    def halo_export(self, side: str) -> np.ndarray:
        """The n_ghost interior rows of the next stage's input next to exchange side "+y"/"-y":
        shape (4, n_ghost, ni), rows in increasing j."""
        g = self.cfg.ghost_layers()
        rows = np.empty((4, g, self.cfg.ni))  # C order: [field][row][column]
        _check(self.L.cato_gpu_halo_export(self.h, SIDES.index(side), _c_ptr(rows)), self.h,
               "halo_export")
        return rows

    def halo_import(self, side: str, rows: np.ndarray) -> None:
        """Write the ghost rows beyond exchange side "+y"/"-y" of the next stage's input."""
        g = self.cfg.ghost_layers()
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        if rows.shape != (4, g, self.cfg.ni):
            raise ValueError(f"halo rows {rows.shape} != {(4, g, self.cfg.ni)}")
        _check(self.L.cato_gpu_halo_import(self.h, SIDES.index(side), _c_ptr(rows)), self.h,
               "halo_import")

    def run(self, t_end: float, max_iterations: int = -1) -> int:
        """The main.f90:138-198 time loop (CFL dt each step, no last-step trim) on the device.
        Returns the number of steps; raises CatoError on a fluid error code."""
        steps = ctypes.c_int64()
        t = ctypes.c_double()
        ec = ctypes.c_int32()
        _check(self.L.cato_gpu_run(self.h, int(max_iterations), float(t_end), ctypes.byref(steps),
                                   ctypes.byref(t), ctypes.byref(ec)), self.h, "run")
        if ec.value:
            raise CatoError(ec.value, f"after {steps.value} steps at t={t.value}")
        return steps.value

    def run_timed(self, n_steps: int, per_kernel: bool = False):
        """Exactly n_steps CFL steps on the device, timed with CUDA events on the handle's
        stream.  Returns (total_ms, per-kernel-slot ms or None)."""
        total = ctypes.c_float()
        n = ctypes.c_int32()
        _check(self.L.cato_gpu_launches_per_step(self.h, ctypes.byref(n)), self.h)
        ks = (ctypes.c_float * n.value)() if per_kernel else None
        rc = self.L.cato_gpu_run_timed(self.h, int(n_steps), ctypes.byref(total), ks,
                                       n.value if per_kernel else 0)
        _check(rc, self.h, "run_timed")
        return total.value, (list(ks) if per_kernel else None)

    def set_plan(self, threads: int, rows_per_cta: int) -> None:
        _check(self.L.cato_gpu_set_plan(self.h, int(threads), int(rows_per_cta)), self.h, "plan")

    def get_plan(self) -> tuple[int, int]:
        t, r = ctypes.c_int32(), ctypes.c_int32()
        _check(self.L.cato_gpu_get_plan(self.h, ctypes.byref(t), ctypes.byref(r)), self.h)
        return t.value, r.value

    def set_kernel_variant(self, variant: int) -> None:
        """FP64 stage kernel register budget: 0 (compiler's choice), 1 (<= 128 registers) or
        2 (<= 85)."""
        _check(self.L.cato_gpu_set_kernel_variant(self.h, int(variant)), self.h, "variant")

    def get_kernel_variant(self) -> int:
        v = ctypes.c_int32()
        _check(self.L.cato_gpu_get_kernel_variant(self.h, ctypes.byref(v)), self.h)
        return v.value

    def tune(self, steps: int = 2) -> tuple[int, float]:
        """Autotune plan and kernel variant on the live state (cato_gpu_tune).  The candidates
        run real CFL steps, bit-identical whichever runs them.  Returns (steps taken, the
        fastest candidate's ms per step); raises CatoError on a fluid error."""
        n, ms = ctypes.c_int32(), ctypes.c_float()
        rc = self.L.cato_gpu_tune(self.h, int(steps), ctypes.byref(n), ctypes.byref(ms))
        _check(rc, self.h, f"tune (after {n.value} steps)")
        return n.value, ms.value

    def launches_per_step(self) -> int:
        n = ctypes.c_int32()
        _check(self.L.cato_gpu_launches_per_step(self.h, ctypes.byref(n)), self.h)
        return n.value

    def profile_step(self) -> list:
        """One CFL step with per-kernel CUDA-event times (ms): [step control, stage 1, ...]."""
        n = self.launches_per_step()
        ks = (ctypes.c_float * n)()
        got = ctypes.c_int32()
        _check(self.L.cato_gpu_profile_step(self.h, ks, n, ctypes.byref(got)), self.h, "profile")
        return list(ks)[: got.value]

    def state(self, names=("rho", "rho_u", "rho_v", "rho_E", "u", "v", "p", "cs")) -> dict:
        """Download conserved and derived fields (halo-padded, ghosts zero)."""
        all_names = ("rho", "rho_u", "rho_v", "rho_E", "u", "v", "p", "cs")
        out = {k: (_field(self.cfg) if k in names else None) for k in all_names}
        _check(self.L.cato_gpu_download(self.h, *(_lib.ptr(out[k]) for k in all_names), self.ld),
               self.h, "download")
        return {k: v for k, v in out.items() if v is not None}

    def conservation_sums(self) -> np.ndarray:
        """Interior totals of rho, rho u, rho v, rho E times the cell volume (FP64, deterministic)."""
        out = np.zeros(4)
        _check(self.L.cato_gpu_conservation_sums(self.h, _lib.ptr(out)), self.h,
               "conservation_sums")
        return out

    def set_step_options(self, keep_step_start: bool = False, allow_subcycle: bool = False,
                         subcycle_tolerance: float = 1e-3) -> None:
        """[time] allow_subcycle / subcycle_error_tolerance (subcycle_check,
        mod_fluid.f90:856-887: SSP steps repeat with dt / 10 while a convergence norm exceeds
        the tolerance), and keeping U^n of every step so that :meth:`convergence` also covers
        rk(m,n) steps (the residual history)."""
        _check(self.L.cato_gpu_set_step_options(self.h, int(bool(keep_step_start)),
                                                 int(bool(allow_subcycle)),
                                                 float(subcycle_tolerance)),
               self.h, "set_step_options")

    def convergence(self) -> np.ndarray:
        """calculate_convergence (mod_fluid.f90:1162-1205) of the last step:
        [rho, rho u, rho v, rho E] relative L2 change from the first to the last stage."""
        out = np.zeros(4)
        _check(self.L.cato_gpu_convergence(self.h, _lib.ptr(out)), self.h, "convergence")
        return out

    def t(self):
        """Time derivative of the current state (fluid_t%t, mod_fluid.f90:460-516)."""
        s = self.state(("rho", "u", "v", "p"))
        fs = FluxSolver(self.cfg)
        if getattr(self, "nodes", None) is not None:
            fs.set_rectilinear(*self.nodes)
        if getattr(self, "bc_table", None) is not None:
            fs.set_bc_table(*self.bc_table)
        fs.set_time(self.time, self.iteration)
        return fs.solve(s["rho"], s["u"], s["v"], s["p"])


class FluxSolver(_Handle):
    """flux_solver_t%solve for the configured flux / limiter / boundary conditions."""

    def solve(self, rho, u, v, p, dt: float = 0.0):
        """Returns (d_rho_dt, d_rho_u_dt, d_rho_v_dt, d_rho_E_dt), halo-padded with zero ghosts.
        The boundary conditions are written into the ghosts of rho/u/v/p when they are
        Fortran-ordered float64 arrays of the halo-padded shape (intent(inout))."""
        prims = [_as_field(self.cfg, a) for a in (rho, u, v, p)]
        outs = [_field(self.cfg) for _ in range(4)]
        _check(self.L.cato_gpu_solve(self.h, *(_lib.ptr(a) for a in prims),
                                     *(_lib.ptr(a) for a in outs), self.ld), self.h, "solve")
        for src, dst in zip(prims, (rho, u, v, p)):
            if src is not dst and isinstance(dst, np.ndarray) and dst.shape == src.shape:
                dst[...] = src
        return tuple(outs)


class MusclInterpolator(_Handle):
    """interpolate_edge_values(q) -> (i_edges(2, -1:ni, 0:nj), j_edges(2, 0:ni, -1:nj))."""

    def interpolate_edge_values(self, q):
        q = _as_field(self.cfg, q)
        ni, nj = self.cfg.ni, self.cfg.nj
        ie = np.zeros((2, ni + 2, nj + 1), order="F")
        je = np.zeros((2, ni + 1, nj + 2), order="F")
        _check(self.L.cato_gpu_interpolate_edges(self.h, _lib.ptr(q), self.ld, _lib.ptr(ie),
                                                 _lib.ptr(je)), self.h, "interpolate_edge_values")
        return ie, je
