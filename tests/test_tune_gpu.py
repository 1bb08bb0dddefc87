"""Autotuning of the stage kernel (cato_gpu_tune) and the FP64 kernel variants: the solution is
the same whichever plan or register budget runs the steps, so tuning on the live state leaves
the result bit-identical to an untuned run of the same number of steps."""
import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import Fluid

pytestmark = pytest.mark.gpu


def _cfg(flux, limiter, precision="fp64", n=96):
    return SchemeConfig(ni=n, nj=n + 8, dx=1.0 / n, dy=1.0 / n, flux_solver=flux,
                        limiter=limiter, gamma=1.4, cfl=0.4, precision=precision,
                        integration_strategy="ssp_rk3")


@pytest.mark.parametrize("flux,limiter", [("HLLC", "van_leer"), ("Roe", "superbee"),
                                          ("SLAU", "MLP5")])
def test_variants_bit_identical(flux, limiter):
    cfg = _cfg(flux, limiter)
    prims = random_prims(cfg, np.random.default_rng(3))
    out = []
    for variant in (0, 1, 2):
        f = Fluid(cfg).initialize(*prims)
        f.set_kernel_variant(variant)
        assert f.get_kernel_variant() == variant
        f.run_timed(4)
        out.append(f.state(("rho", "rho_u", "rho_v", "rho_E")))
        f.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
        assert np.array_equal(out[0][k], out[2][k]), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tune_matches_untuned_run(precision):
    cfg = _cfg("HLLC", "van_leer", precision=precision)
    prims = random_prims(cfg, np.random.default_rng(5))
    f = Fluid(cfg).initialize(*prims)
    taken, ms = f.tune(1)
    # small grid: one plan fits (256-wide strips exceed it, half of 8 rows is 8), with the three
    # FP64 register budgets
    assert taken == (3 if precision == "fp64" else 1) and ms > 0.0
    assert f.get_kernel_variant() in (0, 1, 2)
    threads, rows = f.get_plan()
    assert 64 <= threads <= 256 and rows >= 1
    f.run_timed(2)
    tuned = f.state(("rho", "rho_u", "rho_v", "rho_E"))
    f.close()
    g = Fluid(cfg).initialize(*prims)
    g.run_timed(taken + 2)
    plain = g.state(("rho", "rho_u", "rho_v", "rho_E"))
    g.close()
    for k in tuned:
        assert np.array_equal(tuned[k], plain[k]), k


def test_variant_rejects_bad_values():
    cfg = _cfg("HLLC", "van_leer")
    f = Fluid(cfg)
    with pytest.raises(Exception):
        f.set_kernel_variant(3)
    f.close()
