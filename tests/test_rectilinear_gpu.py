"""Rectilinear grids on the device against the oracle: per-cell volume, edge lengths and
min_dx/min_dy from the node coordinates (grid_block_2d.f90:370-387, quad_cell.f90:69-229) in the
flux divergence, the CFL step and the conservation totals."""
import itertools

import numpy as np
import pytest

from conftest import interior, random_prims
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import CatoError, Fluid, FluxSolver
from test_rectilinear_cpu import stretched_nodes

pytestmark = pytest.mark.gpu

BCS = {
    "zg_sym": {"+x": "zero_gradient", "-x": "zero_gradient", "+y": "symmetry", "-y": "symmetry"},
    "per": {"+x": "periodic", "-x": "periodic", "+y": "periodic", "-y": "periodic"},
    "out": {"+x": "outlet", "-x": "symmetry", "+y": "zero_gradient", "-y": "symmetry"},
}


def _cfg(flux, limiter, bc, ni=83, nj=47, **kw):
    return SchemeConfig(ni=ni, nj=nj, dx=1.0 / ni, dy=0.7 / nj, flux_solver=flux, limiter=limiter,
                        bc=BCS[bc], gamma=1.4, cfl=0.4, outflow_ambient_pressure=0.9, **kw)


def _nodes(cfg, seed):
    return stretched_nodes(cfg.ni, 1.0, seed), stretched_nodes(cfg.nj, 0.7, seed + 1, ratio=4.0)


CASES = list(itertools.product(["AUSMPW+", "SLAU2", "Roe", "HLLC", "M-AUSMPW+"],
                               ["minmod", "van_leer", "MLP3", "MLP5"]))


@pytest.mark.parametrize("flux,limiter", CASES)
def test_solve_bitexact(oracle, cato_lib, flux, limiter):
    bc = ["zg_sym", "per", "out"][CASES.index((flux, limiter)) % 3]
    cfg = _cfg(flux, limiter, bc)
    nodes = _nodes(cfg, CASES.index((flux, limiter)))
    prims = random_prims(cfg, np.random.default_rng(5))
    ref_in = [a.copy(order="F") for a in prims]
    gpu_in = [a.copy(order="F") for a in prims]
    ref = oracle.solve(cfg, *ref_in, nodes=nodes)
    got = FluxSolver(cfg).set_rectilinear(*nodes).solve(*gpu_in)
    for k in range(4):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=f"d/dt var {k}")
        np.testing.assert_array_equal(gpu_in[k], ref_in[k], err_msg=f"BC ghosts var {k}")


@pytest.mark.parametrize("rk,flux", [("ssp_rk3", "AUSMPW+"), ("ssp_rk2", "SD-SLAU"),
                                     ("rk(2,4)", "HLLC"), ("ssp_rk3", "AUSM+-up")])
def test_steps_bitexact(oracle, cato_lib, rk, flux):
    cfg = _cfg(flux, "MLP3", "zg_sym", ni=70, nj=41, integration_strategy=rk)
    nodes = _nodes(cfg, 11)
    prims = random_prims(cfg, np.random.default_rng(3))
    ref = oracle.OracleFluid(cfg)
    ref.set_rectilinear(*nodes)
    ref.set_primitive(*prims)
    gpu = Fluid(cfg).set_rectilinear(*nodes).initialize(*prims)
    assert gpu.get_timestep() == ref.get_timestep()
    for _ in range(5):
        assert ref.integrate() == 0
        gpu.integrate()
    a, b = ref.state(), gpu.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E", "u", "v", "p", "cs"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    assert gpu.time == ref.time
    if not rk.startswith("rk("):
        np.testing.assert_allclose(gpu.convergence(), ref.convergence(), rtol=1e-12, atol=0)
    got, want = gpu.conservation_sums(), ref.conservation_sums()
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13 * np.abs(want).max())


def test_time_derivative_uses_the_grid(oracle, cato_lib):
    """fluid_t%t on a rectilinear Fluid builds its flux solver on the same nodes."""
    cfg = _cfg("SLAU", "MLP3", "zg_sym", ni=40, nj=30)
    nodes = _nodes(cfg, 2)
    prims = random_prims(cfg, np.random.default_rng(8))
    gpu = Fluid(cfg).set_rectilinear(*nodes).initialize(*prims)
    s = gpu.state(("rho", "u", "v", "p"))
    want = oracle.solve(cfg, *(s[k].copy(order="F") for k in ("rho", "u", "v", "p")),
                        nodes=nodes)
    got = gpu.t()
    for k in range(4):
        np.testing.assert_array_equal(interior(cfg, got[k]), interior(cfg, want[k]))


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_mixed_steps_close(oracle, cato_lib, precision):
    cfg = _cfg("HLLC", "van_leer", "zg_sym", ni=70, nj=41, integration_strategy="ssp_rk3")
    nodes = _nodes(cfg, 21)
    prims = random_prims(cfg, np.random.default_rng(13))
    ref = oracle.OracleFluid(cfg)
    ref.set_rectilinear(*nodes)
    ref.set_primitive(*prims)
    cfg_m = _cfg("HLLC", "van_leer", "zg_sym", ni=70, nj=41, integration_strategy="ssp_rk3",
                 precision=precision)
    gpu = Fluid(cfg_m).set_rectilinear(*nodes).initialize(*prims)
    for _ in range(6):
        assert ref.integrate() == 0
        gpu.integrate()
    # FP32 arithmetic (and FP32 reciprocal cell widths) carries ~1e-7 relative error per stage;
    # double-float ~1e-13
    tol = {"mixed": 2e-6, "mixed_df": 1e-10}[precision]
    assert abs(gpu.time - ref.time) <= tol * ref.time
    a, b = ref.state(), gpu.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        x, y = interior(cfg, a[k]), interior(cfg, b[k])
        l1 = np.abs(y - x).sum() / np.abs(x).sum()
        assert l1 <= tol, (k, l1)


def test_back_to_uniform_and_bad_nodes(oracle, cato_lib):
    cfg = _cfg("AUSMPW+", "minmod", "zg_sym", ni=32, nj=24)
    prims = random_prims(cfg, np.random.default_rng(4))
    f = Fluid(cfg)
    xs, ys = _nodes(cfg, 3)
    f.set_rectilinear(xs, ys)
    f.set_rectilinear(None, None)
    f.initialize(*prims)
    ref = oracle.OracleFluid(cfg)
    ref.set_primitive(*prims)
    assert f.get_timestep() == ref.get_timestep()
    bad = xs.copy()
    bad[5] = np.nan
    with pytest.raises(CatoError):
        f.set_rectilinear(bad, ys)
    with pytest.raises(CatoError):
        f.set_rectilinear(xs, ys[::-1].copy())
    with pytest.raises(ValueError):
        f.set_rectilinear(xs[:-1], ys)
