"""Rectilinear grids in the oracle: per-cell quad_cell_t metrics from node coordinates
(grid_block_2d.f90:370-387, quad_cell.f90:69-229), checked against the uniform path and
against the telescoping of the flux divergence."""
import numpy as np
import pytest

from conftest import interior, random_prims
from fvleg_2d_gb300.config import SchemeConfig

PERIODIC = {"+x": "periodic", "-x": "periodic", "+y": "periodic", "-y": "periodic"}
ZG = {"+x": "zero_gradient", "-x": "zero_gradient", "+y": "symmetry", "-y": "symmetry"}


def stretched_nodes(n, length, seed, ratio=2.5):
    """Strictly increasing nodes 0..length whose widths vary smoothly by `ratio` plus noise."""
    rng = np.random.default_rng(seed)
    s = (np.arange(n) + 0.5) / n
    w = 1.0 + (ratio - 1.0) * 0.5 * (1.0 + np.sin(2 * np.pi * s + seed)) + 0.1 * rng.random(n)
    x = np.concatenate([[0.0], np.cumsum(w)])
    return x * (length / x[-1])


def _cfg(ni, nj, flux="AUSMPW+", limiter="minmod", bc=ZG, rk="ssp_rk3"):
    return SchemeConfig(ni=ni, nj=nj, dx=1.0 / 64, dy=1.0 / 32, flux_solver=flux, limiter=limiter,
                        bc=bc, gamma=1.4, cfl=0.4, integration_strategy=rk)


def test_power_of_two_nodes_equal_uniform(oracle):
    """Nodes k * dx with a power-of-two dx are exact, so every per-cell metric equals the
    uniform one and the rectilinear solve is the uniform solve bit for bit."""
    cfg = _cfg(40, 24, flux="SLAU", limiter="MLP3")
    prims = random_prims(cfg, np.random.default_rng(1))
    xs, ys = np.arange(cfg.ni + 1) / 64.0, np.arange(cfg.nj + 1) / 32.0
    a = oracle.solve(cfg, *[p.copy(order="F") for p in prims])
    b = oracle.solve(cfg, *[p.copy(order="F") for p in prims], nodes=(xs, ys))
    for k in range(4):
        np.testing.assert_array_equal(a[k], b[k])
    f, g = oracle.OracleFluid(cfg), oracle.OracleFluid(cfg)
    g.set_rectilinear(xs, ys)
    f.set_primitive(*prims)
    g.set_primitive(*prims)
    assert f.get_timestep() == g.get_timestep()
    for _ in range(3):
        f.integrate()
        g.integrate()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(f.state()[k], g.state()[k])
    np.testing.assert_allclose(f.conservation_sums(), g.conservation_sums(), rtol=1e-14)


def test_cell_metrics_are_the_quad_cell_metrics(oracle):
    xs, ys = stretched_nodes(7, 1.3, 2), stretched_nodes(5, 0.9, 3)
    i, j = 4, 2
    m = oracle.quad_metrics([xs[i], xs[i + 1], xs[i + 1], xs[i]],
                            [ys[j], ys[j], ys[j + 1], ys[j + 1]])
    w, h = xs[i + 1] - xs[i], ys[j + 1] - ys[j]
    assert m["volume"] == w * h
    np.testing.assert_array_equal(m["edge_lengths"], [w, h, w, h])
    assert (m["min_dx"], m["min_dy"]) == (w, h)
    np.testing.assert_array_equal(m["edge_norm_vectors"], [[0, -1], [1, 0], [0, 1], [-1, 0]])


def test_stretched_periodic_box_conserves(oracle):
    """The divergence telescopes on any rectilinear grid: the volume-weighted totals of mass
    and energy of a periodic box stay constant up to rounding."""
    cfg = _cfg(48, 36, flux="HLLC", limiter="van_leer", bc=PERIODIC)
    f = oracle.OracleFluid(cfg)
    f.set_rectilinear(stretched_nodes(48, 1.0, 4), stretched_nodes(36, 0.75, 5))
    f.set_primitive(*random_prims(cfg, np.random.default_rng(6)))
    t0 = f.conservation_sums()
    for _ in range(10):
        assert f.integrate() == 0
    t1 = f.conservation_sums()
    for k in (0, 3):
        assert abs(t1[k] - t0[k]) <= 1e-12 * abs(t0[k]), (k, t0[k], t1[k])


def test_timestep_uses_the_smallest_cells(oracle):
    cfg = _cfg(32, 16)
    prims = random_prims(cfg, np.random.default_rng(7))
    xs, ys = stretched_nodes(32, 0.5, 8, ratio=6.0), stretched_nodes(16, 0.5, 9, ratio=6.0)
    f = oracle.OracleFluid(cfg)
    f.set_rectilinear(xs, ys)
    f.set_primitive(*prims)
    s = f.state()
    u, v, cs = (interior(cfg, s[k]) for k in ("u", "v", "cs"))
    dx, dy = np.diff(xs)[:, None], np.diff(ys)[None, :]
    expect = (cfg.cfl / (((np.abs(u) + cs) / dx) + ((np.abs(v) + cs) / dy))).min()
    assert f.get_timestep() == expect


def test_bad_nodes_rejected(oracle):
    cfg = _cfg(8, 6)
    f = oracle.OracleFluid(cfg)
    xs, ys = stretched_nodes(8, 1.0, 1), stretched_nodes(6, 1.0, 2)
    bad = xs.copy()
    bad[3] = bad[2]
    with pytest.raises(ValueError):
        f.set_rectilinear(bad, ys)
    prims = random_prims(cfg, np.random.default_rng(1))
    with pytest.raises(RuntimeError):
        oracle.solve(cfg, *prims, nodes=(xs, ys[::-1].copy()))
