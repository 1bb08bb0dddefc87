"""Global diagnostics on the device: conservation totals (FP64, deterministic reduction) and the
reference's per-step L2 convergence norms (calculate_convergence, mod_fluid.f90:1162-1205),
both against the oracle."""
import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import CatoError, Fluid

pytestmark = pytest.mark.gpu

PERIODIC = {"+x": "periodic", "-x": "periodic", "+y": "periodic", "-y": "periodic"}
MIXED_BC = {"+x": "zero_gradient", "-x": "zero_gradient", "+y": "symmetry", "-y": "symmetry"}


def _cfg(rk, precision="fp64", bc=MIXED_BC, flux="SLAU", limiter="MLP3", ni=97, nj=61):
    return SchemeConfig(ni=ni, nj=nj, dx=1.0 / ni, dy=0.8 / nj, flux_solver=flux, limiter=limiter,
                        bc=bc, gamma=1.4, cfl=0.4, integration_strategy=rk, precision=precision)


def _pair(oracle, cfg, seed, steps):
    prims = random_prims(cfg, np.random.default_rng(seed))
    f = Fluid(cfg).initialize(*prims)
    o = oracle.OracleFluid(cfg)
    o.set_primitive(*prims)
    for _ in range(steps):
        f.integrate()
        o.integrate()
    return f, o


@pytest.mark.parametrize("rk", ["ssp_rk2", "ssp_rk3"])
def test_fp64_convergence_and_sums_match_oracle(oracle, cato_lib, rk):
    f, o = _pair(oracle, _cfg(rk), 11, 4)
    # the FP64 states are bit-identical; only the summation order differs
    np.testing.assert_allclose(f.convergence(), o.convergence(), rtol=1e-12, atol=0)
    got, ref = f.conservation_sums(), o.conservation_sums()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13 * scale)


def test_sums_are_deterministic(cato_lib):
    cfg = _cfg("ssp_rk3", ni=517, nj=389)
    f = Fluid(cfg).initialize(*random_prims(cfg, np.random.default_rng(3)))
    f.integrate()
    a, b = f.conservation_sums(), f.conservation_sums()
    assert a.tobytes() == b.tobytes()
    c1, c2 = f.convergence(), f.convergence()
    assert c1.tobytes() == c2.tobytes()


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_df"])
def test_periodic_box_conserves_mass_and_energy(cato_lib, precision):
    cfg = _cfg("ssp_rk3", precision=precision, bc=PERIODIC, flux="HLLC", limiter="van_leer")
    f = Fluid(cfg).initialize(*random_prims(cfg, np.random.default_rng(5)))
    t0 = f.conservation_sums()
    for _ in range(25):
        f.integrate()
    t1 = f.conservation_sums()
    # the flux divergence telescopes up to rounding (and its 1e-14 relative cut); the mixed path
    # rounds each cell's FP32 increment, so its totals drift by ~eps_f32 * |increment| per step
    tol = {"fp64": 1e-12, "mixed": 1e-8, "mixed_df": 1e-11}[precision]
    for k in (0, 3):
        assert abs(t1[k] - t0[k]) <= tol * abs(t0[k]), (k, t0[k], t1[k])


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
@pytest.mark.parametrize("rk", ["ssp_rk2", "ssp_rk3", "rk(2,4)"])
def test_mixed_convergence_close_to_oracle(oracle, cato_lib, rk, precision):
    if rk.startswith("rk("):
        pytest.skip("every precision keeps the FP64 layout: rk(m,n) overwrites U_0 (tested above)")
    cfg = _cfg(rk, precision=precision)
    f, o = _pair(oracle, cfg, 21, 3)
    # FP32 flux arithmetic: the stage change itself carries ~1e-6 relative error; double-float
    # ~1e-12
    rtol = {"mixed": 2e-4, "mixed_df": 1e-6}[precision]
    np.testing.assert_allclose(f.convergence(), o.convergence(), rtol=rtol, atol=1e-12)


def test_convergence_state_errors(cato_lib):
    cfg = _cfg("ssp_rk2")
    f = Fluid(cfg).initialize(*random_prims(cfg, np.random.default_rng(1)))
    with pytest.raises(CatoError):
        f.convergence()  # no step since the upload
    f.integrate()
    f.convergence()
    cfg = _cfg("rk(1,3)")
    f = Fluid(cfg).initialize(*random_prims(cfg, np.random.default_rng(1)))
    f.integrate()
    with pytest.raises(CatoError):
        f.convergence()  # FP64 rk(m,n) overwrites U_0 in place
