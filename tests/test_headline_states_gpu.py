"""GPU parity on the benchmarked schemes' own initial states, the Roe entropy fix under every
boundary-condition set, and the reference's error codes on poisoned and failing states.

FP64 path: bit-identical to the oracle (state, dt sequence, time), checked with exact equality.
"""
import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300 import ic
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import Fluid, FluxSolver
from test_parity_gpu import BCS, _run_pair

pytestmark = pytest.mark.gpu

CONSERVED = ("rho", "rho_u", "rho_v", "rho_E")


def _assert_same_state(ref, gpu, keys=CONSERVED + ("u", "v", "p", "cs")):
    a, b = ref.state(), gpu.state()
    for k in keys:
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    assert gpu.time == ref.time
    assert gpu.iteration == ref.iteration


def test_quadrant_256_steps_bitexact(oracle, cato_lib):
    """The four-quadrant Riemann problem of the single-grid benchmark (HLLC, van Leer,
    SSP-RK3, CFL 0.4, transmissive boundaries) on 256^2: 40 CFL steps identical to the oracle.
    Whole quadrants start with exactly zero velocity components."""
    cfg, prims = ic.riemann_quadrant(256)
    ref, gpu = _run_pair(oracle, cfg, prims, 40)
    _assert_same_state(ref, gpu)


def test_kelvin_helmholtz_256_harten_steps_bitexact(oracle, cato_lib):
    """The Kelvin-Helmholtz shear layer of the roofline benchmark (Roe with the Harten entropy
    fix, superbee, SSP-RK3, CFL 0.4, periodic x / symmetry y) on 256^2: 30 CFL steps identical to
    the oracle, including the periodic/symmetry corners."""
    cfg, prims = ic.kelvin_helmholtz(256, roe_entropy_fix="harten")
    ref, gpu = _run_pair(oracle, cfg, prims, 30)
    _assert_same_state(ref, gpu)


@pytest.mark.parametrize("bc", sorted(BCS))
@pytest.mark.parametrize("limiter", ["superbee", "MLP3"])
def test_roe_harten_solve_every_bc_set_bitexact(oracle, cato_lib, bc, limiter):
    """flux_solver_t%solve with Roe + the Harten entropy fix (roe_solver.fypp:529-536): residuals
    and BC-filled ghosts identical to the oracle for every boundary-condition set."""
    cfg = SchemeConfig(ni=77, nj=45, dx=1.0 / 77, dy=0.6 / 45, flux_solver="Roe", limiter=limiter,
                       bc=BCS[bc], gamma=1.4, cfl=0.4, roe_entropy_fix="harten",
                       outflow_ambient_pressure=0.7)
    prims = random_prims(cfg, np.random.default_rng(sorted(BCS).index(bc) + 40))
    ref_in = [a.copy(order="F") for a in prims]
    gpu_in = [a.copy(order="F") for a in prims]
    ref = oracle.solve(cfg, *ref_in)
    got = FluxSolver(cfg).solve(*gpu_in)
    for k in range(4):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=f"d/dt var {k}")
        np.testing.assert_array_equal(gpu_in[k], ref_in[k], err_msg=f"BC ghosts var {k}")


# ---- error codes (error.f90:6-9): NEG_DENSITY = 1, NEG_PRESSURE = 2, NANS_FOUND = 3 ----------

def _upload(cfg, prims):
    """(GPU upload code, GPU fluid or None)."""
    from fvleg_2d_gb300.fluid import CatoError

    try:
        return 0, Fluid(cfg).initialize(*prims)
    except CatoError as e:
        return e.code, None


@pytest.mark.parametrize("var", ["rho", "u", "v", "p"])
def test_nan_in_uploaded_state_gives_nans_found(oracle, cato_lib, var):
    """A NaN in one interior cell of rho, u, v or p: the upload accepts it (minval skips NaNs,
    mod_fluid.f90:352-360) and the next step reports NANS_FOUND, as the reference's first stage
    assignment does (check_for_nans, mod_fluid.f90:718-721)."""
    cfg = SchemeConfig(ni=40, nj=24, dx=1.0 / 40, dy=1.0 / 40, flux_solver="AUSMPW+",
                       limiter="minmod", bc=BCS["zg_sym"], gamma=1.4, cfl=0.4)
    prims = random_prims(cfg, np.random.default_rng(5))
    g = cfg.ghost_layers()
    prims[["rho", "u", "v", "p"].index(var)][g + 17, g + 9] = np.nan
    ref = oracle.OracleFluid(cfg)
    code_ref = ref.set_primitive(*prims)
    code_gpu, gpu = _upload(cfg, prims)
    assert code_gpu == code_ref == 0
    ec_ref = ref.integrate(1e-4)
    _, ec_gpu = gpu.integrate(1e-4)
    assert ec_gpu == ec_ref == 3


@pytest.mark.parametrize("poison,code", [("rho", 1), ("p", 2), ("both", 2), ("rho_zero", 1)])
def test_negative_uploaded_state_codes(oracle, cato_lib, poison, code):
    """Negative (or zero) density or pressure in the uploaded state: initialize_from_hdf5 refuses
    pressure below tiny first, then density below tiny (mod_fluid.f90:352-360)."""
    cfg = SchemeConfig(ni=40, nj=24, dx=1.0 / 40, dy=1.0 / 40, flux_solver="HLLC",
                       limiter="van_leer", bc=BCS["per"], gamma=1.4, cfl=0.4)
    prims = random_prims(cfg, np.random.default_rng(6))
    g = cfg.ghost_layers()
    if poison in ("rho", "both"):
        prims[0][g + 30, g + 3] = -0.2
    if poison in ("p", "both"):
        prims[3][g + 5, g + 20] = -1e-3
    if poison == "rho_zero":
        prims[0][g + 1, g + 1] = 0.0
    code_ref = oracle.OracleFluid(cfg).set_primitive(*prims)
    code_gpu, _ = _upload(cfg, prims)
    assert code_gpu == code_ref == code


# random-circle states (the serving workload's initial states, 48 x 32) that fail in the
# reference scheme itself, found with the oracle: (flux, limiter, seed, expected code)
FAILING = [("AUSMPW+", "minmod", 1, 2), ("AUSM+-up", "minmod", 1, 1),
           ("AUSMPW+", "minmod", 2, 3), ("Roe", "minmod", 16, 1)]


@pytest.mark.parametrize("flux,limiter,seed,code", FAILING)
def test_failing_runs_report_the_oracles_code(oracle, cato_lib, flux, limiter, seed, code):
    """States whose own evolution produces a negative density, a negative pressure or a NaN:
    the GPU stops at the same step with the same code, bit-identical up to that step."""
    cfg, prims = ic.random_circles(48, 32, np.random.default_rng(seed), flux_solver=flux,
                                   limiter=limiter)
    ref = oracle.OracleFluid(cfg)
    assert ref.set_primitive(*prims) == 0
    gpu = Fluid(cfg).initialize(*prims)
    for n in range(150):
        dt_ref = ref.get_timestep()
        ec_ref = ref.integrate(dt_ref)
        dt_gpu, ec_gpu = gpu.integrate()
        assert dt_gpu == dt_ref, n
        assert ec_gpu == ec_ref, n
        if ec_ref:
            break
    assert ec_ref == code
    a, b = ref.state(), gpu.state()
    for k in CONSERVED:
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
