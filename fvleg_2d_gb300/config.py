"""Scheme configuration: the ``cato_config`` C struct and the reference's deck names.

The names accepted here are the reference's own ``.ini`` values:

* ``[scheme] flux_solver``  -- ``src/lib/fluid/mod_fluid.f90:223-238`` (plus ``AUSM+-up`` and
  ``HLLC``, which the reference declares but cannot run);
* ``[scheme] limiter``      -- ``src/lib/spatial_reconstruction/muscl_factory.f90:69-83``;
* ``[time] integration_strategy`` -- ``src/lib/fluid/mod_fluid.f90:424-446``;
* ``[boundary_conditions]`` -- ``src/lib/boundary_conditions/bc_factory.f90:39-66``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

FLUX_IDS = {
    "AUSMPW+": 0,
    "SLAU": 1,
    "SLAU2": 2,
    "SD-SLAU": 3,
    "SD-SLAU2": 4,
    "Roe": 5,
    "AUSM+-up": 6,
    "HLLC": 7,
    "M-AUSMPW+": 8,
}
LIMITER_IDS = {"minmod": 0, "superbee": 1, "van_leer": 2, "vanleer": 2, "MLP3": 3, "MLP5": 4}
RK_IDS = {
    "ssp_rk2": 0,
    "ssp_rk3": 1,
    "ssp_rk33": 1,
    "rk(1,3)": 2,
    "rk(1,4)": 3,
    "rk(1,5)": 4,
    "rk(2,3)": 5,
    "rk(2,4)": 6,
    "rk(2,5)": 7,
}
# bc_factory.f90:46-59 names
BC_IDS = {"zero_gradient": 0, "symmetry": 1, "mirror": 1, "reflection": 1, "periodic": 2,
          "outlet": 3, "outflow": 3, "pressure_input": 4, "exchange": 5}
PRECISION_IDS = {"fp64": 0, "mixed": 1, "mixed_df": 2}
# side order of cato_config.bc: the reference's application order (flux_solver.f90:165-183)
SIDES = ("+x", "+y", "-x", "-y")

# status codes (include/cato_gpu.h); 1..3 are the reference's error codes (src/lib/error.f90:6-9)
CATO_OK = 0
CATO_NEG_DENSITY = 1
CATO_NEG_PRESSURE = 2
CATO_NANS_FOUND = 3
CATO_ERR_CONFIG = 10
CATO_ERR_OOM = 11
CATO_ERR_CUDA = 12
CATO_ERR_ARG = 13
CATO_ERR_TIMEOUT = 14
CATO_ERR_STATE = 15
CATO_ERR_CAPACITY = 16
CATO_ERR_BC_INPUT = 17
STATUS_NAMES = {
    0: "ALL_OK",
    1: "NEG_DENSITY",
    2: "NEG_PRESSURE",
    3: "NANS_FOUND",
    10: "ERR_CONFIG",
    11: "ERR_OOM",
    12: "ERR_CUDA",
    13: "ERR_ARG",
    14: "ERR_TIMEOUT",
    15: "ERR_STATE",
    16: "ERR_CAPACITY",
    17: "ERR_BC_INPUT",
}


class CatoConfig(ctypes.Structure):
    """Mirror of ``struct cato_config`` in ``include/cato_gpu.h``."""

    _fields_ = [
        ("ni", ctypes.c_int32),
        ("nj", ctypes.c_int32),
        ("n_ghost", ctypes.c_int32),
        ("flux", ctypes.c_int32),
        ("limiter", ctypes.c_int32),
        ("rk", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 4),
        ("apply_low_mach_fix", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("roe_entropy_fix", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("gamma", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("harten_delta", ctypes.c_double),
        ("ausm_beta", ctypes.c_double),
        ("ausm_kp", ctypes.c_double),
        ("ausm_ku", ctypes.c_double),
        ("ausm_sigma", ctypes.c_double),
        ("bc_pressure", ctypes.c_double),
        ("bc_density", ctypes.c_double),
    ]


@dataclass
class SchemeConfig:
    """A grid instance's scheme, in the reference's vocabulary.

    Defaults are the reference deck defaults (``src/lib/io/mod_input.f90:34-148``) except the
    boundary conditions, which the caller always states.
    """

    ni: int
    nj: int
    dx: float
    dy: float
    flux_solver: str = "AUSMPW+"
    limiter: str = "minmod"
    integration_strategy: str = "ssp_rk2"
    bc: dict = field(default_factory=lambda: {s: "periodic" for s in SIDES})
    gamma: float = 5.0 / 3.0
    cfl: float = 0.1
    apply_low_mach_fix: bool = True
    precision: str = "fp64"
    roe_entropy_fix: str = "reference"  # or "harten"
    harten_delta: float = 0.1
    ausm_beta: float = 1.0 / 8.0
    ausm_kp: float = 0.25
    ausm_ku: float = 0.75
    ausm_sigma: float = 1.0
    outflow_ambient_pressure: float = 0.0  # [boundary_conditions], for 'outflow' sides
    # constant target of a 'pressure_input' side (non-dimensional; a table replaces both,
    # Fluid.set_bc_table).  The reference keeps the outflow pressure and this one in the same
    # variable, the outflow value winning when both BCs are present (mod_input.f90:366-390).
    constant_bc_pressure: float = 0.0
    bc_density: float = 0.0
    n_ghost: int | None = None

    def ghost_layers(self) -> int:
        if self.n_ghost is not None:
            return self.n_ghost
        # mod_input.f90:320-338: MLP5 needs 3 ghost layers, everything else 2
        return 3 if self.limiter == "MLP5" else 2

    def to_c(self) -> CatoConfig:
        try:
            c = CatoConfig()
            c.ni, c.nj = int(self.ni), int(self.nj)
            c.n_ghost = self.ghost_layers()
            c.flux = FLUX_IDS[self.flux_solver]
            c.limiter = LIMITER_IDS[self.limiter]
            c.rk = RK_IDS[self.integration_strategy]
            for k, side in enumerate(SIDES):
                c.bc[k] = BC_IDS[self.bc[side]]
            c.apply_low_mach_fix = 1 if self.apply_low_mach_fix else 0
            c.precision = PRECISION_IDS[self.precision]
            c.roe_entropy_fix = {"reference": 0, "harten": 1}[self.roe_entropy_fix]
        except KeyError as exc:  # the reference stops with "Invalid flux solver ..." etc.
            raise ValueError(f"unknown scheme name: {exc}") from None
        c.gamma, c.cfl, c.dx, c.dy = self.gamma, self.cfl, self.dx, self.dy
        c.harten_delta = self.harten_delta
        c.ausm_beta, c.ausm_kp = self.ausm_beta, self.ausm_kp
        c.ausm_ku, c.ausm_sigma = self.ausm_ku, self.ausm_sigma
        outlet = any(BC_IDS[self.bc[s]] == 3 for s in SIDES)
        c.bc_pressure = self.outflow_ambient_pressure if outlet else self.constant_bc_pressure
        c.bc_density = self.bc_density
        return c

    @property
    def halo_shape(self) -> tuple[int, int]:
        """Shape of one halo-padded field, Fortran order (i, j)."""
        g = self.ghost_layers()
        return (self.ni + 2 * g, self.nj + 2 * g)


SOURCE_GEOMETRY_IDS = {"uniform": 0, "constant_xy": 1, "1d_gaussian": 2, "decay": 3}


class CatoEnergySource(ctypes.Structure):
    """Mirror of ``struct cato_energy_source`` in ``include/cato_gpu.h``."""

    _fields_ = [
        ("geometry", ctypes.c_int32),
        ("gaussian_order", ctypes.c_int32),
        ("constant_value", ctypes.c_double),
        ("multiplier", ctypes.c_double),
        ("xlo", ctypes.c_double),
        ("xhi", ctypes.c_double),
        ("ylo", ctypes.c_double),
        ("yhi", ctypes.c_double),
        ("fwhm_x", ctypes.c_double),
        ("fwhm_y", ctypes.c_double),
    ]


@dataclass
class EnergySource:
    """An energy source term ([source_terms], ``source_t`` of ``mod_source.f90``), in the
    reference's non-dimensional units.  ``table = (time, value, critical_density)`` replaces
    the constant value (scaled as read_input_file scales it)."""

    geometry: str = "uniform"
    constant_value: float = 0.0
    multiplier: float = 1.0
    xlo: float = 0.0
    xhi: float = 0.0
    ylo: float = 0.0
    yhi: float = 0.0
    fwhm_x: float = 0.0
    fwhm_y: float = 0.0
    gaussian_order: int = 1
    table: tuple | None = None

    def to_c(self) -> CatoEnergySource:
        if self.geometry not in SOURCE_GEOMETRY_IDS:
            raise ValueError(f"Unsupported geometry type {self.geometry!r}, must be one of "
                             f"{sorted(SOURCE_GEOMETRY_IDS)}")
        c = CatoEnergySource()
        c.geometry = SOURCE_GEOMETRY_IDS[self.geometry]
        c.gaussian_order = int(self.gaussian_order)
        c.constant_value, c.multiplier = self.constant_value, self.multiplier
        c.xlo, c.xhi, c.ylo, c.yhi = self.xlo, self.xhi, self.ylo, self.yhi
        c.fwhm_x, c.fwhm_y = self.fwhm_x, self.fwhm_y
        return c
