"""Input decks: the reference's ``.ini`` format read into the hot path's configuration.

Follows ``input_t%read_from_ini`` (``src/lib/io/mod_input.f90:194-445``): the same sections,
keys and defaults (``mod_input.f90:34-155``).  Values may be quoted with single or double quotes,
``;`` and ``#`` start comments, logicals are ``true``/``.true.``/``t`` (any case) and reals may
use a Fortran ``d`` exponent.

A deck whose initial conditions come from a file (``read_from_file = true``) takes its grid and
state from that file in pycato's layout (:mod:`.icfile`; ``.npz`` stands in for HDF5 when
h5py is not installed): :func:`run_deck` loads it.  A deck with ``read_from_file = false`` is
complete: its uniform initial state and grid come from the deck (``[initial_conditions] init_*``,
``[grid] ni_nodes ... ymax``).
"""
from __future__ import annotations

import configparser
import os
from dataclasses import dataclass, field

import numpy as np

from .config import BC_IDS, FLUX_IDS, LIMITER_IDS, RK_IDS, SchemeConfig

_TRUE = {"true", ".true.", "t", "yes", "on", "1"}
_FALSE = {"false", ".false.", "f", "no", "off", "0"}


class DeckError(ValueError):
    """An invalid deck (the reference stops with error_msg in the same situations)."""


def _strip(v: str) -> str:
    v = v.strip()
    if len(v) >= 2 and v[0] == v[-1] and v[0] in "'\"":
        v = v[1:-1]
    return v.strip()


def _real(v: str) -> float:
    return float(_strip(v).replace("d", "e").replace("D", "e"))


def _logical(v: str) -> bool:
    s = _strip(v).lower()
    if s in _TRUE:
        return True
    if s in _FALSE:
        return False
    raise DeckError(f"not a logical: {v!r}")


@dataclass
class Deck:
    # [general]
    title: str = ""
    units: str = "cgs"
    # [reference_state]
    non_dimensionalize: bool = True
    reference_length: float = 1.0
    reference_density: float = 1.0
    reference_velocity: float = 1.0
    # [time]
    max_time: float = 1.0
    initial_delta_t: float = 0.0
    use_constant_delta_t: bool = False
    cfl: float = 0.1
    integration_strategy: str = ""
    max_iterations: int = 2**31 - 1
    allow_subcycle: bool = False
    subcycle_error_tolerance: float = 1e-3
    # [physics]
    polytropic_index: float = 5.0 / 3.0
    # [scheme]
    flux_solver: str = "AUSMPW+"
    spatial_reconstruction: str = "MUSCL"
    limiter: str = "minmod"
    apply_low_mach_fix: bool = True
    # [ausm] (read only for AUSM+-up, mod_input.f90:262-267)
    ausm_beta: float = 1.0 / 8.0
    ausm_pressure_diffusion_coeff: float = 0.25
    ausm_pressure_flux_coeff: float = 0.75
    ausm_sonic_point_sigma: float = 1.0
    # [initial_conditions]
    read_from_file: bool = True
    initial_condition_file: str = ""
    init_density: float = 0.0
    init_x_velocity: float = 0.0
    init_y_velocity: float = 0.0
    init_pressure: float = 0.0
    # [grid]
    n_ghost_layers: int = 2
    grid_type: str = "2d_regular"
    ni_nodes: int = 0
    nj_nodes: int = 0
    xmin: float = 0.0
    xmax: float = 0.0
    ymin: float = 0.0
    ymax: float = 0.0
    # [boundary_conditions]
    bc: dict = field(default_factory=lambda: {s: "periodic" for s in ("+x", "-x", "+y", "-y")})
    outflow_ambient_pressure: float = 0.0
    # pressure_input sides (mod_input.f90:366-382); the outflow pressure and the constant
    # pressure are one variable there (constant_bc_pressure_value), the outflow key read last
    apply_constant_bc_pressure: bool = False
    bc_density: float = 0.0
    constant_bc_pressure_value: float = 0.0
    bc_pressure_input_file: str = ""
    bc_pressure_scale_factor: float = 1.0
    # [source_terms] (mod_input.f90:394-427)
    enable_source_terms: bool = False
    source_geometry: str = ""
    apply_constant_source: bool = False
    source_file: str = ""
    source_term_type: str = ""
    constant_source_value: float = 0.0
    source_scale_factor: float = 1.0
    energy_deposition_critical_density: float = 0.1
    source_xlo: float = 0.0
    source_xhi: float = 0.0
    source_ylo: float = 0.0
    source_yhi: float = 0.0
    source_center_x: float = 0.0
    source_center_y: float = 0.0
    source_gaussian_fwhm_x: float = 0.0
    source_gaussian_fwhm_y: float = 0.0
    source_gaussian_order: int = 1
    # [io]
    contour_interval_dt: float = 0.1
    contour_format: str = "xdmf"

    def scheme(self, ni: int | None = None, nj: int | None = None, dx: float | None = None,
               dy: float | None = None, precision: str = "fp64") -> SchemeConfig:
        """The hot path's configuration of this deck on an ni x nj grid of dx x dy cells (from
        the deck's own grid keys when the initial state is not read from a file)."""
        if ni is None:
            ni, nj, dx, dy = self.grid()
        strategy = self.integration_strategy
        if strategy not in RK_IDS:
            raise DeckError(f"integration_strategy {strategy!r} is not supported "
                            f"(one of {sorted(RK_IDS)}; 'ssp_rk43' is a no-op in the reference)")
        if self.flux_solver not in FLUX_IDS:
            raise DeckError(f"flux_solver {self.flux_solver!r} is not supported ({sorted(FLUX_IDS)})")
        if self.limiter not in LIMITER_IDS:
            raise DeckError(f"limiter {self.limiter!r} is not supported ({sorted(LIMITER_IDS)})")
        for side, name in self.bc.items():
            if name not in BC_IDS:
                raise DeckError(f"boundary condition {name!r} at {side} is not supported")
        f = nondim_factors(self)
        return SchemeConfig(
            ni=int(ni), nj=int(nj), dx=float(dx), dy=float(dy), flux_solver=self.flux_solver,
            limiter=self.limiter, integration_strategy=strategy, bc=dict(self.bc),
            gamma=self.polytropic_index, cfl=self.cfl,
            apply_low_mach_fix=self.apply_low_mach_fix, precision=precision,
            ausm_beta=self.ausm_beta, ausm_kp=self.ausm_pressure_diffusion_coeff,
            ausm_ku=self.ausm_pressure_flux_coeff, ausm_sigma=self.ausm_sonic_point_sigma,
            # outlet_bc.f90:55 and pressure_input_bc.f90:82-89 (the density there is scaled
            # with density_to_dim)
            outflow_ambient_pressure=self.outflow_ambient_pressure * f["press_to_nondim"],
            constant_bc_pressure=self.constant_bc_pressure_value * f["press_to_nondim"],
            bc_density=self.bc_density * f["density_to_dim"],
            n_ghost=self.n_ghost_layers)

    def grid(self) -> tuple[int, int, float, float]:
        """(ni, nj, dx, dy) of a deck-defined uniform grid: nodes - 1 cells per direction."""
        if self.read_from_file:
            raise DeckError("the grid comes from the initial condition file; pass ni, nj, dx, dy")
        if self.ni_nodes < 2 or self.nj_nodes < 2:
            raise DeckError("[grid] ni_nodes and nj_nodes must be >= 2")
        ni, nj = self.ni_nodes - 1, self.nj_nodes - 1
        return ni, nj, (self.xmax - self.xmin) / ni, (self.ymax - self.ymin) / nj

    def initial_primitives(self, cfg: SchemeConfig) -> list[np.ndarray]:
        """The uniform initial state of [initial_conditions] init_* (halo-padded, ghosts 0)."""
        if self.read_from_file:
            raise DeckError("the initial state comes from a file: upload its primitives")
        g = cfg.ghost_layers()
        out = []
        for val in (self.init_density, self.init_x_velocity, self.init_y_velocity,
                    self.init_pressure):
            a = np.zeros(cfg.halo_shape, order="F")
            a[g:g + cfg.ni, g:g + cfg.nj] = val
            out.append(a)
        return out


def _ghost_layers_for(limiter: str) -> int:
    """mod_input.f90:318-338: the ghost layers an edge interpolation scheme needs."""
    if limiter in ("minmod", "superbee", "van_leer", "vanleer", "none", "TVD2", "TVD3", "MLP3",
                   "eMLP3"):
        return 2
    if limiter in ("TVD5", "MLP5", "eMLP5"):
        return 3
    raise DeckError("Unknown edge interpolation scheme, must be one of the following: "
                    "'TVD2', 'TVD3', 'TVD5', 'MLP3', or 'MLP5'")


def parse_deck(text: str) -> Deck:
    """Parse the text of an input deck."""
    cp = configparser.ConfigParser(inline_comment_prefixes=(";", "#"),
                                   comment_prefixes=(";", "#"), interpolation=None, strict=False)
    cp.read_string(text)

    def get(sec, key, conv=_strip, default=None, required=False):
        if cp.has_option(sec, key):
            return conv(cp.get(sec, key))
        if required:
            raise DeckError(f"[{sec}] {key} is required")
        return default

    d = Deck()
    d.title = get("general", "title", default="")
    d.units = get("general", "units", default="cgs")
    d.non_dimensionalize = get("reference_state", "non_dimensionalize", _logical, True)
    if d.non_dimensionalize:
        d.reference_length = get("reference_state", "reference_length", _real, 1.0)
        d.reference_density = get("reference_state", "reference_density", _real, 1.0)
        d.reference_velocity = get("reference_state", "reference_velocity", _real, 1.0)
    d.max_time = get("time", "max_time", _real, required=True)
    d.initial_delta_t = get("time", "initial_delta_t", _real, 0.0)
    d.use_constant_delta_t = get("time", "use_constant_delta_t", _logical, False)
    d.cfl = get("time", "cfl", _real, 0.1)
    d.integration_strategy = get("time", "integration_strategy", required=True)
    d.max_iterations = get("time", "max_iterations", lambda v: int(_real(v)), 2**31 - 1)
    d.allow_subcycle = get("time", "allow_subcycle", _logical, False)
    d.subcycle_error_tolerance = get("time", "subcycle_error_tolerance", _real, 1e-3)
    d.polytropic_index = get("physics", "polytropic_index", _real, required=True)
    d.flux_solver = get("scheme", "flux_solver", required=True)
    if d.flux_solver == "AUSM+-up":
        d.ausm_beta = get("ausm", "beta", _real, 1.0 / 8.0)
        d.ausm_pressure_diffusion_coeff = get("ausm", "pressure_diffusion_coeff", _real, 0.25)
        d.ausm_pressure_flux_coeff = get("ausm", "pressure_flux_coeff", _real, 0.75)
        d.ausm_sonic_point_sigma = get("ausm", "sonic_point_sigma", _real, 1.0)
    d.spatial_reconstruction = get("scheme", "spatial_reconstruction", default="MUSCL")
    d.limiter = get("scheme", "limiter", default="minmod")
    d.apply_low_mach_fix = get("scheme", "apply_low_mach_fix", _logical, True)
    d.read_from_file = get("initial_conditions", "read_from_file", _logical, True)
    if d.read_from_file:
        d.initial_condition_file = get("initial_conditions", "initial_condition_file",
                                       required=True)
    d.init_density = get("initial_conditions", "init_density", _real, 0.0)
    d.init_x_velocity = get("initial_conditions", "init_x_velocity", _real, 0.0)
    d.init_y_velocity = get("initial_conditions", "init_y_velocity", _real, 0.0)
    d.init_pressure = get("initial_conditions", "init_pressure", _real, 0.0)
    need = _ghost_layers_for(d.limiter)
    d.n_ghost_layers = get("grid", "n_ghost_layers", lambda v: int(_real(v)), need)
    if d.n_ghost_layers != need:
        raise DeckError("The number of required ghost cell layers doesn't match the edge "
                        "interpolation order")
    d.grid_type = get("grid", "grid_type", default="2d_regular")
    if not d.read_from_file:
        d.ni_nodes = get("grid", "ni_nodes", lambda v: int(_real(v)), required=True)
        d.nj_nodes = get("grid", "nj_nodes", lambda v: int(_real(v)), required=True)
        d.xmin = get("grid", "xmin", _real, required=True)
        d.xmax = get("grid", "xmax", _real, required=True)
        d.ymin = get("grid", "ymin", _real, required=True)
        d.ymax = get("grid", "ymax", _real, required=True)
    for side, key in (("+x", "plus_x"), ("-x", "minus_x"), ("+y", "plus_y"), ("-y", "minus_y")):
        d.bc[side] = get("boundary_conditions", key, default="periodic")
    if "pressure_input" in d.bc.values():
        d.apply_constant_bc_pressure = get("boundary_conditions", "apply_constant_bc_pressure",
                                           _logical, False)
        d.bc_density = get("boundary_conditions", "bc_density", _real, 0.0)
        if d.apply_constant_bc_pressure:
            d.constant_bc_pressure_value = get("boundary_conditions",
                                               "constant_bc_pressure_value", _real, required=True)
        else:
            d.bc_pressure_input_file = get("boundary_conditions", "bc_pressure_input_file",
                                           required=True)
        d.bc_pressure_scale_factor = get("boundary_conditions", "bc_pressure_scale_factor",
                                         _real, 1.0)
    if "outflow" in d.bc.values():
        d.outflow_ambient_pressure = get("boundary_conditions", "outflow_ambient_pressure", _real,
                                         required=True)
        d.constant_bc_pressure_value = d.outflow_ambient_pressure
    d.enable_source_terms = get("source_terms", "enable_source_terms", _logical, False)
    if d.enable_source_terms:
        d.source_geometry = get("source_terms", "geometry", required=True)
        d.apply_constant_source = get("source_terms", "apply_constant_source", _logical, False)
        d.source_file = get("source_terms", "source_file", required=True)
        d.source_term_type = get("source_terms", "source_term_type", required=True)
        d.constant_source_value = get("source_terms", "constant_source_value", _real, 0.0)
        d.source_scale_factor = get("source_terms", "source_scale_factor", _real, 1.0)
        d.energy_deposition_critical_density = get(
            "source_terms", "energy_deposition_critical_density", _real, 0.1)
        if d.source_geometry == "constant_xy":
            for k in ("xlo", "xhi", "ylo", "yhi"):
                setattr(d, "source_" + k, get("source_terms", k, _real, required=True))
        elif d.source_geometry in ("1d_gaussian", "2d_gaussian"):
            d.source_center_x = get("source_terms", "center_x", _real, 0.0)
            d.source_center_y = get("source_terms", "center_y", _real, 0.0)
            d.source_gaussian_fwhm_x = get("source_terms", "gaussian_fwhm_x", _real, 0.0)
            d.source_gaussian_fwhm_y = get("source_terms", "gaussian_fwhm_y", _real, 0.0)
            d.source_gaussian_order = get("source_terms", "gaussian_order",
                                          lambda v: int(_real(v)), 1)
    d.contour_format = get("io", "format", default=get("io", "contour_format", default="xdmf"))
    d.contour_interval_dt = get("io", "contour_interval_dt", _real, 0.1)
    return d


def read_deck(path: str) -> Deck:
    """Read an input deck file (``cato.x input.ini``'s argument)."""
    with open(path) as f:
        return parse_deck(f.read())


def load_initial_condition(deck: Deck, base_dir: str = "."):
    """The deck's initial-condition file (pycato layout, see :mod:`.icfile`) in the reference's
    non-dimensional units."""
    from .icfile import read_ic

    path = deck.initial_condition_file
    if not os.path.isabs(path):
        path = os.path.join(base_dir, path)
    return read_ic(path, deck.n_ghost_layers, deck.reference_length, deck.reference_density,
                   deck.reference_velocity, deck.non_dimensionalize)


def nondim_factors(deck: Deck) -> dict:
    """The scale factors of ``set_refrence_quantities`` (``non_dimensional.f90:95-135``), all 1
    without non-dimensionalization."""
    names = ("len_to_nondim", "t_to_nondim", "density_to_nondim", "density_to_dim",
             "vel_to_nondim", "press_to_nondim", "pow_to_nondim")
    if not deck.non_dimensionalize:
        return dict.fromkeys(names, 1.0)
    L, R, V = deck.reference_length, deck.reference_density, deck.reference_velocity
    t_ref = L / V
    press_ref = R * (V * V)
    pow_ref = R * (V * V) / t_ref
    return {"len_to_nondim": 1.0 / L, "t_to_nondim": 1.0 / t_ref, "density_to_nondim": 1.0 / R,
            "density_to_dim": R, "vel_to_nondim": 1.0 / V, "press_to_nondim": 1.0 / press_ref,
            "pow_to_nondim": 1.0 / pow_ref}


def t_to_nondim(deck: Deck) -> float:
    """1 / t_ref with t_ref = reference_length / reference_velocity
    (``non_dimensional.f90:95-118``); 1 without non-dimensionalization."""
    return nondim_factors(deck)["t_to_nondim"]


def read_bc_pressure_table(deck: Deck, base_dir: str = "."):
    """The pressure-input table of ``bc_pressure_input_file`` as read_pressure_input reads it
    (``pressure_input_bc.f90:92-181``): an optional first line starting with '#', then rows of
    time [s], pressure [barye], density [g/cc] (list-directed, reading stops at the first row
    that does not parse); scaled to time x t_to_nondim, pressure x press_to_nondim x
    bc_pressure_scale_factor and density x density_to_nondim x bc_pressure_scale_factor."""
    a = _read_table3(deck.bc_pressure_input_file, base_dir, "Pressure input file")
    f = nondim_factors(deck)
    scale = deck.bc_pressure_scale_factor
    return (a[:, 0] * f["t_to_nondim"], (a[:, 1] * f["press_to_nondim"]) * scale,
            (a[:, 2] * f["density_to_nondim"]) * scale)


def energy_source(deck: Deck, base_dir: str = "."):
    """The deck's energy source term as an EnergySource (new_source, mod_source.f90:63-125:
    positions x len_to_nondim; read_input_file :127-258: time x t_to_nondim, value x
    pow_to_nondim, critical density x density_to_nondim; the constant value is used as given);
    None when source terms are off."""
    from .config import EnergySource, SOURCE_GEOMETRY_IDS

    if not deck.enable_source_terms:
        return None
    if deck.source_term_type != "energy":
        raise DeckError(f"source_term_type {deck.source_term_type!r} is not supported ('energy')")
    if deck.source_geometry not in SOURCE_GEOMETRY_IDS:
        raise DeckError("Unsupported geometry type, must be one of ['uniform', 'constant_xy', "
                        "'1d_gaussian']")
    f = nondim_factors(deck)
    L = f["len_to_nondim"]
    table = None
    if not deck.apply_constant_source:
        a = _read_table3(deck.source_file, base_dir, "source input file")
        table = (a[:, 0] * f["t_to_nondim"], a[:, 1] * f["pow_to_nondim"],
                 a[:, 2] * f["density_to_nondim"])
    return EnergySource(
        geometry=deck.source_geometry, constant_value=deck.constant_source_value,
        multiplier=deck.source_scale_factor, xlo=deck.source_xlo * L, xhi=deck.source_xhi * L,
        ylo=deck.source_ylo * L, yhi=deck.source_yhi * L,
        fwhm_x=deck.source_gaussian_fwhm_x * L, fwhm_y=deck.source_gaussian_fwhm_y * L,
        gaussian_order=deck.source_gaussian_order, table=table)


def _read_table3(name: str, base_dir: str, what: str) -> np.ndarray:
    """Rows of three reals after an optional '#' header line, list-directed: reading stops at
    the first row that does not parse (read_pressure_input / read_input_file)."""
    path = name if os.path.isabs(name) else os.path.join(base_dir, name)
    if not os.path.exists(path):
        raise DeckError(f"{what} '{path}' not found")
    rows = []
    with open(path) as fh:
        lines = fh.read().splitlines()
    if lines and lines[0].lstrip().startswith("#"):
        lines = lines[1:]
    for line in lines:
        parts = line.replace(",", " ").split()
        if not parts:
            continue
        try:
            row = [_real(x) for x in parts[:3]]
        except ValueError:
            break
        if len(row) < 3:
            break
        rows.append(row)
    if len(rows) < 2:
        raise DeckError(f"{path}: the table needs at least two rows")
    return np.array(rows, dtype=np.float64)


def fortran_es(x: float, w: int, d: int) -> str:
    """Fortran ESw.d editing: one digit before the point, d after, a two-digit exponent with
    its E (three digits without it beyond 99), right-justified in w characters."""
    import math

    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    mant, exp = f"{x:.{d}E}".split("E")
    e = int(exp)
    return (f"{mant}E{e:+03d}" if abs(e) < 100 else f"{mant}{e:+04d}").rjust(w)


class RunHistory:
    """The reference's per-run files: ``residual_hist.csv`` (fluid_t%initialize truncates it and
    write_residual_history appends a line per step, mod_fluid.f90:244-246, 1207-1223),
    ``timing.csv`` (timer_t%log_time, mod_timing.f90:57-94) and ``timing_summary.yaml``
    (timer_t%output_stats, :104-127), written into ``directory``."""

    def __init__(self, directory: str, t_to_dim: float):
        import os
        import time

        os.makedirs(directory, exist_ok=True)
        self.dir = directory
        self.t_to_dim = t_to_dim
        self.res = open(os.path.join(directory, "residual_hist.csv"), "w")
        self.res.write("iteration,time,dt,rho,rho_u,rho_v,rho_E\n")
        self.tim = open(os.path.join(directory, "timing.csv"), "w")
        self.tim.write("iteration, elapsed_wall_time[sec], elapsed_cpu_time[sec], timestep[sec]\n")
        self.wall0, self.cpu0 = time.perf_counter(), time.process_time()

    def residual(self, iteration: int, time: float, dt: float, norms) -> None:
        vals = [time * self.t_to_dim, dt * self.t_to_dim] + [float(x) for x in norms]
        self.res.write(f"{iteration}," + "".join(fortran_es(v, 16, 6) + "," for v in vals) + "\n")
        self.res.flush()

    def timing(self, iteration: int, timestep: float) -> None:
        import time

        vals = [time.perf_counter() - self.wall0, time.process_time() - self.cpu0, timestep]
        self.tim.write(f"{iteration}" + "".join(", " + fortran_es(v, 14, 4) for v in vals) + "\n")

    def close(self) -> None:
        import os
        import time

        wall, cpu = time.perf_counter() - self.wall0, time.process_time() - self.cpu0
        with open(os.path.join(self.dir, "timing_summary.yaml"), "w") as f:
            for label, v in (("wall time [s]", wall), ("wall time [m]", wall / 60.0),
                             ("wall time [hr]", wall / 3600.0), ("CPU time [s]", cpu),
                             ("CPU time [m]", cpu / 60.0), ("CPU time [hr]", cpu / 3600.0)):
                f.write(f"Total elapsed {label}:{fortran_es(v, 10, 3)}\n")
        self.res.close()
        self.tim.close()


def main_loop(deck: Deck, fluid, step, results_dir: str | None = None) -> int:
    """The time loop of ``main.f90:95-198`` (no restart, no start-up period) around a fluid:
    ``step(dt)`` advances one step (``dt`` None: the CFL step) and returns its error code.  The
    loop keeps its own clock: it snaps to the next output time when a step passes it, writes a
    contour the iteration after (``write_contour`` of :mod:`.contour`, when ``results_dir`` is
    given), and stops on that clock.  The first step uses ``initial_delta_t`` when it is set,
    every step when ``use_constant_delta_t``.  With ``results_dir`` it also writes the
    residual history and the timing files there (:class:`RunHistory`).  Returns the iterations
    taken."""
    from .contour import write_contour
    from .fluid import CatoError

    f = nondim_factors(deck)
    interval = deck.contour_interval_dt * f["t_to_nondim"]
    max_time = deck.max_time * f["t_to_nondim"]
    eps = float(np.finfo(np.float64).eps)
    time, iteration = 0.0, 0
    next_output = 0.0 + interval
    hist = None
    if results_dir is not None:
        write_contour(fluid, results_dir, deck, iteration=iteration)
        hist = RunHistory(results_dir, 1.0 / f["t_to_nondim"])
    while time < max_time and iteration < deck.max_iterations:
        fixed = deck.use_constant_delta_t or (iteration == 0 and deck.initial_delta_t > 0.0)
        ec = step(deck.initial_delta_t * f["t_to_nondim"] if fixed else None)
        delta_t = fluid.last_dt
        new_time = fluid.time
        if hist is not None:
            hist.residual(fluid.iteration, new_time, delta_t, fluid.convergence())
        if ec:
            if results_dir is not None:
                write_contour(fluid, results_dir, deck, iteration=iteration)
                hist.close()
            raise CatoError(ec, f"time integration failed at iteration {iteration}")
        if abs(time - next_output) < eps:
            next_output = next_output + interval
            if results_dir is not None:
                write_contour(fluid, results_dir, deck, iteration=iteration)
        if new_time > next_output:
            delta_t = abs(next_output - time)
            new_time = time + delta_t
        time = new_time
        iteration = iteration + 1
        if hist is not None:
            hist.timing(iteration, delta_t)
    if hist is not None:
        hist.close()
    return iteration


def run_deck(deck: Deck, precision: str = "fp64", prims=None, grid=None, base_dir: str = ".",
             results_dir: str | None = None):
    """The main.f90 time loop for a deck: returns (fluid, steps).  A deck that reads its
    initial state from a file loads it (grid included) from ``initial_condition_file`` relative
    to ``base_dir``; alternatively pass that state as ``prims`` (rho, u, v, p, halo-padded) and
    a uniform grid as ``grid=(ni, nj, dx, dy)``.  ``max_time`` is scaled by ``t_to_nondim``
    as in ``main.f90:98``.  With ``results_dir`` (contour output) or a deck-given dt the loop
    runs on the host (:func:`main_loop`); otherwise on the device (``cato_gpu_run``, the same
    loop while no output time falls inside it)."""
    from .fluid import Fluid

    ic = None
    if deck.read_from_file and prims is None:
        ic = load_initial_condition(deck, base_dir)
        grid, prims = ic.scheme_grid(), ic.primitives
    cfg = deck.scheme(*(grid or (None, None, None, None)), precision=precision)
    if prims is None:
        prims = deck.initial_primitives(cfg)
    fluid = Fluid(cfg)
    if ic is not None:
        ic.apply_grid(fluid)
    if "pressure_input" in deck.bc.values() and not deck.apply_constant_bc_pressure:
        fluid.set_bc_table(*read_bc_pressure_table(deck, base_dir))
    src = energy_source(deck, base_dir)
    if src is not None:
        # the source's cell centroids need the node coordinates of the grid
        if ic is not None:
            if ic.uniform is not None:
                fluid.set_rectilinear(ic.x_nodes, ic.y_nodes)
        elif grid is None and not deck.read_from_file:
            fluid.set_rectilinear(deck.xmin + np.arange(cfg.ni + 1) * cfg.dx,
                                  deck.ymin + np.arange(cfg.nj + 1) * cfg.dy)
        fluid.set_energy_source(src)
    if deck.allow_subcycle or results_dir is not None:
        # subcycling, and U^n of every step for the residual history of rk(m,n) steps
        fluid.set_step_options(keep_step_start=results_dir is not None,
                               allow_subcycle=deck.allow_subcycle,
                               subcycle_tolerance=deck.subcycle_error_tolerance)
    fluid.initialize(*prims)
    if results_dir is None and not deck.use_constant_delta_t and not deck.initial_delta_t > 0.0:
        steps = fluid.run(deck.max_time * t_to_nondim(deck), deck.max_iterations)
        return fluid, steps
    return fluid, main_loop(deck, fluid, lambda dt: fluid.integrate(dt)[1], results_dir)
