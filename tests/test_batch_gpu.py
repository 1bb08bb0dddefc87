"""Batched engine: every instance of a batch of uneven grids gives exactly what the same
instance gives alone (single-instance handle, and alone in a batch), with its own dt sequence
and stop condition."""
import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300 import ic
from fvleg_2d_gb300.batch import Batch
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.fluid import Fluid

pytestmark = pytest.mark.gpu


def _instances(precision, n=6, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for k, (nx, ny) in enumerate(ic.batch_sides(n, rng, lo=32, hi=160)):
        cfg, prims = ic.random_circles(nx, ny, rng, precision=precision,
                                       limiter=["MLP5", "MLP5", "MLP5"][k % 3])
        out.append((cfg, prims))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_df"])
def test_batch_instances_match_single_handles(cato_lib, precision):
    insts = _instances(precision)
    steps = [7, 12, 3, 20, 9, 15]
    b = Batch(len(insts), precision=precision, integration_strategy="ssp_rk2")
    b.set_plan(64, 16)
    slots = [b.add(cfg, prims, max_steps=s) for (cfg, prims), s in zip(insts, steps)]
    b.step(40)  # more than any instance needs: finished instances idle
    for slot, (cfg, prims), s in zip(slots, insts, steps):
        q = b.query(slot)
        assert q["iteration"] == s and not q["running"] and q["error_code"] == 0
        f = Fluid(cfg).initialize(*prims)
        for _ in range(s):
            f.integrate()
        ref = f.state(("rho", "rho_u", "rho_v", "rho_E"))
        got = b.state(slot)
        if precision == "mixed":
            # FP32 arithmetic built with FMA contraction: the batch kernel (compiled for 3 CTAs
            # per SM) and the single-grid kernel may contract differently, so they agree to
            # FP32 rounding, not bitwise.  (Alone and in a mix, the batch is bitwise: below.)
            assert abs(f.time - q["time"]) <= 1e-6 * q["time"]
            for k in ref:
                np.testing.assert_allclose(got[k], ref[k], rtol=1e-5, atol=1e-6,
                                           err_msg=f"slot {slot} {k}")
            continue
        assert f.time == q["time"]
        for k in ref:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"slot {slot} {k}")


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_df"])
def test_alone_equals_in_mix(cato_lib, precision):
    insts = _instances(precision, n=5, seed=9)
    mix = Batch(8, precision=precision)
    slots = [mix.add(cfg, prims, max_steps=25) for cfg, prims in insts]
    mix.step(32)
    for slot, (cfg, prims) in zip(slots, insts):
        alone = Batch(1, precision=precision)
        s = alone.add(cfg, prims, max_steps=25)
        alone.step(32)
        a, m = alone.state(s), mix.state(slot)
        for k in a:
            np.testing.assert_array_equal(m[k], a[k])
        alone.close()


def test_batch_t_end_and_removal(cato_lib):
    cfg, prims = ic.sod(ni=100, nj=10)
    b = Batch(4, precision="fp64")
    s0 = b.add(cfg, prims, t_end=0.05)
    s1 = b.add(cfg, prims, t_end=0.1)
    b.step(200)
    q0, q1 = b.query(s0), b.query(s1)
    assert q0["time"] >= 0.05 and q0["time"] - q0["dt"] < 0.05
    assert q1["time"] >= 0.1 and q1["iteration"] > q0["iteration"]
    f = Fluid(cfg).initialize(*prims)
    n = f.run(0.05)
    assert n == q0["iteration"] and f.time == q0["time"]
    b.remove(s0)
    s2 = b.add(cfg, prims, max_steps=3)
    assert s2 == s0
    b.step(5)
    assert b.query(s2)["iteration"] == 3
