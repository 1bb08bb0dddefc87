"""The energy source term on the device against the oracle: the per-step field (deposition
column, table or constant input, geometry) added to the energy equation at every stage."""
import numpy as np
import pytest

from conftest import interior, random_prims
from fvleg_2d_gb300.config import EnergySource, SchemeConfig
from fvleg_2d_gb300.fluid import CatoError, Fluid
from test_source_cpu import SOURCES, TABLE

pytestmark = pytest.mark.gpu

BC = {"+x": "zero_gradient", "-x": "zero_gradient", "+y": "symmetry", "-y": "symmetry"}


def _cfg(rk="ssp_rk3", precision="fp64", ni=67, nj=29):
    return SchemeConfig(ni=ni, nj=nj, dx=1.0 / ni, dy=0.5 / nj, bc=BC, gamma=1.4, cfl=0.4,
                        flux_solver="SLAU", limiter="MLP3", integration_strategy=rk,
                        precision=precision)


def _nodes(cfg):
    w = 0.5 + np.random.default_rng(9).random(cfg.ni)
    xn = np.concatenate([[0.0], np.cumsum(w)])
    return xn / xn[-1], np.linspace(0.0, 0.5, cfg.nj + 1)


def _pair(oracle, cfg, src, rect, t0=0.0, seed=2):
    prims = random_prims(cfg, np.random.default_rng(seed))
    ref = oracle.OracleFluid(SchemeConfig(**{**cfg.__dict__, "precision": "fp64"}))
    gpu = Fluid(cfg)
    if rect:
        ref.set_rectilinear(*_nodes(cfg))
        gpu.set_rectilinear(*_nodes(cfg))
    ref.set_primitive(*prims)
    gpu.initialize(*prims)
    ref.set_time(t0, 0)
    gpu.set_time(t0, 0)
    ref.set_energy_source(src)
    gpu.set_energy_source(src)
    return ref, gpu


@pytest.mark.parametrize("k", range(len(SOURCES)))
@pytest.mark.parametrize("rk", ["ssp_rk2", "ssp_rk3", "rk(2,4)"])
def test_steps_bitexact(oracle, cato_lib, k, rk):
    """Steps starting at t = 0.296 cross the table's 0.3 point; the correctly rounded exp and
    power on both sides."""
    cfg = _cfg(rk)
    with oracle.pow_mode("cr"):
        ref, gpu = _pair(oracle, cfg, SOURCES[k], rect=k % 2 == 0, t0=0.296)
        for _ in range(6):
            assert ref.integrate() == 0
            _, ec = gpu.integrate()
            assert ec == 0
    a, b = ref.state(), gpu.state()
    for key in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(b[key], a[key], err_msg=key)
    assert gpu.time == ref.time


def test_table_end_turns_the_source_off(oracle, cato_lib):
    """Past the table's last time the input is zero (get_desired_source_input)."""
    cfg = _cfg()
    src = EnergySource("uniform", table=(np.array([0.0, 0.01]), np.array([3.0, 3.0]),
                                         np.array([0.0, 0.0])))
    with oracle.pow_mode("cr"):
        ref, gpu = _pair(oracle, cfg, src, rect=False, t0=0.005)
        for _ in range(12):
            assert ref.integrate() == 0
            gpu.integrate()
    assert gpu.time > 0.01
    np.testing.assert_array_equal(gpu.state(("rho_E",))["rho_E"], ref.state()["rho_E"])


def test_run_matches_integrate(cato_lib):
    cfg = _cfg()
    prims = random_prims(cfg, np.random.default_rng(4))
    a = Fluid(cfg).set_energy_source(SOURCES[2]).initialize(*prims)
    b = Fluid(cfg).set_energy_source(SOURCES[2]).initialize(*prims)
    n = a.run(0.05)
    for _ in range(n):
        b.integrate()
    assert a.time == b.time
    np.testing.assert_array_equal(a.state(("rho_E",))["rho_E"], b.state(("rho_E",))["rho_E"])


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_mixed_close(oracle, cato_lib, precision):
    cfg = _cfg(precision=precision)
    with oracle.pow_mode("cr"):
        ref, gpu = _pair(oracle, cfg, SOURCES[4], rect=True, t0=0.1)
        for _ in range(6):
            assert ref.integrate() == 0
            gpu.integrate()
    # SLAU's pressure-difference switches can flip on a 1e-13 difference and move a few cells
    # by ~1e-8, as in the parity tests
    tol = {"mixed": 2e-6, "mixed_df": 1e-9}[precision]
    a, b = ref.state(), gpu.state()
    for key in ("rho", "rho_u", "rho_v", "rho_E"):
        x, y = interior(cfg, a[key]), interior(cfg, b[key])
        assert np.abs(y - x).sum() <= tol * np.abs(x).sum(), key


def test_libm_within_tolerance(oracle, cato_lib):
    """Against the oracle with the reference's libm exp and pow: within the FP64 path's 1e-12
    relative L1."""
    cfg = _cfg()
    ref, gpu = _pair(oracle, cfg, SOURCES[2], rect=True, t0=0.0)
    for _ in range(30):
        assert ref.integrate() == 0
        gpu.integrate()
    a, b = ref.state(), gpu.state()
    for key in ("rho", "rho_u", "rho_v", "rho_E"):
        x, y = interior(cfg, a[key]), interior(cfg, b[key])
        assert np.abs(y - x).sum() <= 1e-12 * np.abs(x).sum(), key


def test_errors(cato_lib):
    f = Fluid(_cfg())
    with pytest.raises(CatoError):
        f.set_energy_source(EnergySource("1d_gaussian", fwhm_x=0.1, fwhm_y=0.1))
    with pytest.raises(CatoError):
        f.set_energy_source(EnergySource("1d_gaussian", fwhm_x=0.1, gaussian_order=0))
    with pytest.raises(CatoError):
        f.set_energy_source(EnergySource("uniform", table=([0.0, 0.0], [1.0, 1.0], [0.0, 0.0])))
    f.set_energy_source(SOURCES[0])
    f.set_energy_source(None)
