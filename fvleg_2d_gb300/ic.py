"""Initial conditions for the benchmark and parity workloads.

Cell centres follow the reference's IC generator (``pycato/generate_initial_grids.py:43-113``:
nodes from ``numpy.linspace`` over the ghost-extended range, centres at node + dx/2).  Fields are
halo-padded Fortran-order float64 arrays, the layout of ``field_2d_t%data``; ghost cells are 0
(the reference only reads the interior of an IC file, ``mod_fluid.f90:339-345``).
"""
from __future__ import annotations

import math

import numpy as np

from .config import SchemeConfig


def node_coordinates(n: int, lo: float, hi: float, ng: int) -> np.ndarray:
    """The n + 1 + 2*ng node coordinates (ghost nodes included), pycato's make_uniform_grid."""
    d = float(hi - lo) / float(n)
    return np.linspace(lo - ng * d, hi + ng * d, (n + 1) + 2 * ng, dtype=np.float64)


def cell_centres(n: int, lo: float, hi: float, ng: int) -> np.ndarray:
    """Centres of the n + 2*ng cells (ghosts included), pycato's make_uniform_grid."""
    d = float(hi - lo) / float(n)
    return node_coordinates(n, lo, hi, ng)[:-1] + d / 2.0


def _fields(cfg: SchemeConfig):
    return [np.zeros(cfg.halo_shape, dtype=np.float64, order="F") for _ in range(4)]


def _interior(cfg: SchemeConfig, a: np.ndarray) -> np.ndarray:
    g = cfg.ghost_layers()
    return a[g:g + cfg.ni, g:g + cfg.nj]


def sod(ni: int = 400, nj: int = 40, **scheme) -> tuple[SchemeConfig, list]:
    """2-D Sod shock tube over [0,1]x[0,0.1] (400x40: dx = dy = 0.0025): x < 0.5 (1,0,0,1),
    else (0.125,0,0,0.1); AUSMPW+, minmod, SSP-RK2, CFL 0.5, gamma 1.4; zero-gradient x,
    symmetry y."""
    opts = dict(flux_solver="AUSMPW+", limiter="minmod", integration_strategy="ssp_rk2",
                gamma=1.4, cfl=0.5,
                bc={"+x": "zero_gradient", "-x": "zero_gradient", "+y": "symmetry",
                    "-y": "symmetry"})
    opts.update(scheme)
    cfg = SchemeConfig(ni=ni, nj=nj, dx=1.0 / ni, dy=0.1 / nj, **opts)
    g = cfg.ghost_layers()
    xc = cell_centres(ni, 0.0, 1.0, g)[g:g + ni]
    rho, u, v, p = _fields(cfg)
    left = (xc < 0.5)[:, None] * np.ones((1, nj), dtype=bool)
    _interior(cfg, rho)[...] = np.where(left, 1.0, 0.125)
    _interior(cfg, p)[...] = np.where(left, 1.0, 0.1)
    return cfg, [rho, u, v, p]


def riemann_quadrant(n: int = 4096, **scheme) -> tuple[SchemeConfig, list]:
    """Four-quadrant 2-D Riemann problem on [0,1]^2 split at (0.5,0.5):
    NE (1.5,0,0,1.5), NW (0.5323,1.206,0,0.3), SW (0.138,1.206,1.206,0.029),
    SE (0.5323,0,1.206,0.3); HLLC, van Leer, SSP-RK3, CFL 0.4, transmissive boundaries."""
    opts = dict(flux_solver="HLLC", limiter="van_leer", integration_strategy="ssp_rk3",
                gamma=1.4, cfl=0.4, bc={s: "zero_gradient" for s in ("+x", "-x", "+y", "-y")})
    opts.update(scheme)
    cfg = SchemeConfig(ni=n, nj=n, dx=1.0 / n, dy=1.0 / n, **opts)
    g = cfg.ghost_layers()
    xc = cell_centres(n, 0.0, 1.0, g)[g:g + n][:, None]
    yc = cell_centres(n, 0.0, 1.0, g)[g:g + n][None, :]
    east, north = xc >= 0.5, yc >= 0.5
    states = {  # (rho, u, v, p)
        (True, True): (1.5, 0.0, 0.0, 1.5),
        (False, True): (0.5323, 1.206, 0.0, 0.3),
        (False, False): (0.138, 1.206, 1.206, 0.029),
        (True, False): (0.5323, 0.0, 1.206, 0.3),
    }
    rho, u, v, p = _fields(cfg)
    for (e, nn), st in states.items():
        mask = (east == e) & (north == nn)
        for arr, val in zip((rho, u, v, p), st):
            _interior(cfg, arr)[mask] = val
    return cfg, [rho, u, v, p]


def kelvin_helmholtz(n: int = 8192, **scheme) -> tuple[SchemeConfig, list]:
    """Kelvin-Helmholtz shear layer on [0,1]^2: |y-0.5| < 0.25 -> rho=2, u=+0.5, else rho=1,
    u=-0.5; p=2.5; v = 0.01 sin(4 pi x); Roe, superbee, SSP-RK3, CFL 0.4; periodic x,
    reflective (symmetry) y."""
    opts = dict(flux_solver="Roe", limiter="superbee", integration_strategy="ssp_rk3",
                gamma=1.4, cfl=0.4,
                bc={"+x": "periodic", "-x": "periodic", "+y": "symmetry", "-y": "symmetry"})
    opts.update(scheme)
    cfg = SchemeConfig(ni=n, nj=n, dx=1.0 / n, dy=1.0 / n, **opts)
    g = cfg.ghost_layers()
    xc = cell_centres(n, 0.0, 1.0, g)[g:g + n][:, None]
    yc = cell_centres(n, 0.0, 1.0, g)[g:g + n][None, :]
    inner = np.abs(yc - 0.5) < 0.25
    rho, u, v, p = _fields(cfg)
    _interior(cfg, rho)[...] = np.where(inner, 2.0, 1.0)
    _interior(cfg, u)[...] = np.where(inner, 0.5, -0.5)
    _interior(cfg, v)[...] = 0.01 * np.sin(4.0 * math.pi * xc) * np.ones_like(yc)
    _interior(cfg, p)[...] = 2.5
    return cfg, [rho, u, v, p]


def random_circles(ni: int, nj: int, rng: np.random.Generator, **scheme):
    """Piecewise-constant state of 4-16 circles over a background (centre U[0,1]^2 scaled to the
    domain, radius U[0.03,0.25]); each region rho~U[0.1,2], p log-uniform [0.01,10],
    u,v~N(0,0.5^2).  Domain [0,ni/max(ni,nj)] x [0,nj/max(ni,nj)] with square cells."""
    opts = dict(flux_solver="SLAU", limiter="MLP5", integration_strategy="ssp_rk2", gamma=1.4,
                cfl=0.5, bc={s: "zero_gradient" for s in ("+x", "-x", "+y", "-y")})
    opts.update(scheme)
    h = 1.0 / max(ni, nj)
    cfg = SchemeConfig(ni=ni, nj=nj, dx=h, dy=h, **opts)
    g = cfg.ghost_layers()
    lx, ly = ni * h, nj * h
    xc = cell_centres(ni, 0.0, lx, g)[g:g + ni][:, None]
    yc = cell_centres(nj, 0.0, ly, g)[g:g + nj][None, :]

    def region_state():
        return (rng.uniform(0.1, 2.0), rng.normal(0.0, 0.5), rng.normal(0.0, 0.5),
                math.exp(rng.uniform(math.log(0.01), math.log(10.0))))

    rho, u, v, p = _fields(cfg)
    bg = region_state()
    for arr, val in zip((rho, u, v, p), bg):
        _interior(cfg, arr)[...] = val
    for _ in range(int(rng.integers(4, 17))):
        cx, cy = rng.uniform(0, lx), rng.uniform(0, ly)
        r = rng.uniform(0.03, 0.25) * max(lx, ly)
        st = region_state()
        mask = (xc - cx) ** 2 + (yc - cy) ** 2 < r * r
        for arr, val in zip((rho, u, v, p), st):
            _interior(cfg, arr)[mask] = val
    return cfg, [rho, u, v, p]


def batch_sides(n: int, rng: np.random.Generator, lo: int = 64, hi: int = 1024,
                aspect=(1.0, 4.0)) -> list[tuple[int, int]]:
    """Uneven grid sizes: side log-uniform in [lo, hi] rounded to 16, aspect ratio U[a0,a1]
    (short side clamped to >= 16)."""
    out = []
    for _ in range(n):
        nx = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))) / 16.0)) * 16
        nx = max(16, nx)
        a = rng.uniform(*aspect)
        ny = max(16, int(round(nx / a / 16.0)) * 16)
        out.append((nx, ny))
    return out
