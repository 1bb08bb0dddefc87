"""The deck's step options through the C-ABI: subcycling (subcycle_check, mod_fluid.f90:856-887)
and the convergence norms of rk(m,n) steps (calculate_convergence(U_0, U_curr),
mod_fluid.f90:970) from the kept step start, against the oracle.

FP64: subcycled steps are bit-identical to the oracle (state, dt of every step, time)."""
import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300 import ic
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import Fluid
from test_parity_gpu import BCS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rk,flux,limiter", [("ssp_rk2", "AUSMPW+", "minmod"),
                                             ("ssp_rk3", "HLLC", "van_leer"),
                                             ("ssp_rk3", "SLAU", "MLP5")])
def test_subcycled_steps_bitexact(oracle, cato_lib, rk, flux, limiter):
    """A tolerance that the first steps of a Sod-like state exceed: those steps repeat with dt/10
    (sometimes more than once), later ones pass; every step's dt, the time and the state equal
    the oracle's."""
    cfg, prims = ic.sod(ni=120, nj=12, flux_solver=flux, limiter=limiter, integration_strategy=rk)
    tol = 2e-3
    ref = oracle.OracleFluid(cfg)
    ref.set_primitive(*prims)
    ref.set_subcycle(True, tol)
    gpu = Fluid(cfg)
    gpu.set_step_options(allow_subcycle=True, subcycle_tolerance=tol)
    gpu.initialize(*prims)
    subcycled = 0
    for n in range(12):
        dt_cfl = gpu.get_timestep()  # the CFL dt of the step's start state
        assert ref.integrate() == 0
        dt_gpu, ec = gpu.integrate()
        assert ec == 0
        assert dt_gpu == ref.dt, n
        subcycled += dt_gpu < dt_cfl
        # the device's reduction order differs from the oracle's: equal to rounding
        np.testing.assert_allclose(gpu.convergence(), ref.convergence(), rtol=1e-12, atol=1e-300)
    assert subcycled >= 1
    assert gpu.time == ref.time
    a, b = ref.state(), gpu.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)


@pytest.mark.parametrize("rk", ["rk(1,3)", "rk(2,4)"])
def test_rk_multistage_convergence_from_the_kept_step_start(oracle, cato_lib, rk):
    cfg = SchemeConfig(ni=64, nj=40, dx=1 / 64, dy=1 / 64, flux_solver="Roe", limiter="superbee",
                       bc=BCS["zg_sym"], gamma=1.4, cfl=0.4, integration_strategy=rk)
    prims = random_prims(cfg, np.random.default_rng(9))
    ref = oracle.OracleFluid(cfg)
    ref.set_primitive(*prims)
    gpu = Fluid(cfg)
    gpu.set_step_options(keep_step_start=True)
    gpu.initialize(*prims)
    for _ in range(4):
        ref.integrate()
        gpu.integrate()
        np.testing.assert_allclose(gpu.convergence(), ref.convergence(), rtol=1e-12, atol=1e-300)
    a, b = ref.state(), gpu.state()
    np.testing.assert_array_equal(b["rho"], a["rho"])


def test_run_with_subcycling_matches_the_oracle_loop(oracle, cato_lib):
    """cato_gpu_run takes its steps from the host when subcycling: same step count and time as
    the oracle's time loop."""
    cfg, prims = ic.sod(ni=80, nj=8)
    ref = oracle.OracleFluid(cfg)
    ref.set_primitive(*prims)
    ref.set_subcycle(True, 5e-3)
    n_ref = ref.run(0.01)
    gpu = Fluid(cfg)
    gpu.set_step_options(allow_subcycle=True, subcycle_tolerance=5e-3)
    gpu.initialize(*prims)
    assert gpu.run(0.01) == n_ref
    assert gpu.time == ref.time
    np.testing.assert_array_equal(gpu.state()["rho"], ref.state()["rho"])
