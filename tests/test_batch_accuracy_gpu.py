"""Accuracy of the mixed precisions on the batched configuration (random circles, SLAU + MLP5,
SSP-RK2, CFL 0.5, 500 steps): every instance's final density against its FP64 run.

The bound is the accuracy target of the mixed-precision batched form, relative L1 density error
<= 1e-6, for the double-float path on every instance that finishes in both precisions.  Some
random-circle flows are
dynamically unstable: the FP64 run itself, started from the same state perturbed by 1e-13
(relative, per cell), drifts from the unperturbed FP64 run by up to ~1e-5 after 500 steps, so
no arithmetic that is not bit-identical to FP64 can stay within 1e-6 of it there.  For such an
instance the test bounds the double-float error by 30x the FP64 run's own drift under that
perturbation instead.
"""
import dataclasses

import numpy as np
import pytest

from fvleg_2d_gb300 import ic
from fvleg_2d_gb300.batch import Batch

pytestmark = pytest.mark.gpu

STEPS = 500


def _instances(n=32, seed=77):
    rng = np.random.default_rng(seed)
    sides = ic.batch_sides(n, rng, lo=64, hi=256)
    return [ic.random_circles(nx, ny, rng) for nx, ny in sides]


def _run(insts, precision, perturb=0.0):
    b = Batch(len(insts), precision=precision)
    prng = np.random.default_rng(5)
    slots = []
    for cfg, prims in insts:
        p = [a.copy(order="F") for a in prims]
        if perturb:
            for a in p:
                a *= 1.0 + perturb * prng.standard_normal(a.shape)
        slots.append(b.add(dataclasses.replace(cfg, precision=precision), p, max_steps=STEPS))
    b.step(STEPS)
    out = []
    for (cfg, _), s in zip(insts, slots):
        g = cfg.ghost_layers()
        out.append((b.query(s)["error_code"], b.state(s)["rho"][g:-g, g:-g].copy()))
    b.close()
    return out


def _rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def test_mixed_df_density_error_on_32_batched_instances(cato_lib):
    insts = _instances()
    ref = _run(insts, "fp64")
    got = _run(insts, "mixed_df")
    pert = None
    compared = 0
    for i, ((c64, r64), (cdf, rdf)) in enumerate(zip(ref, got)):
        if c64 or cdf:
            # a run the reference scheme itself stops: both precisions must stop
            assert c64 and cdf, (i, c64, cdf)
            continue
        compared += 1
        err = _rel_l1(rdf, r64)
        if err <= 1e-6:
            continue
        if pert is None:
            pert = _run(insts, "fp64", perturb=1e-13)
        drift = _rel_l1(pert[i][1], r64)
        assert err <= 30 * drift, (i, err, drift)
    assert compared >= 24


def test_mixed_density_error_on_32_batched_instances(cato_lib):
    """FP32 reconstruction and flux with the FP64 stage accumulation: relative L1 density error
    within 1e-3 on every instance that finishes in both precisions (the FP32 flux error recurs
    every step; measured median ~2e-6, largest ~2e-4 on the full batched configuration)."""
    insts = _instances()
    ref = _run(insts, "fp64")
    got = _run(insts, "mixed")
    for i, ((c64, r64), (c32, r32)) in enumerate(zip(ref, got)):
        if c64 or c32:
            assert c64 and c32, (i, c64, c32)
            continue
        assert _rel_l1(r32, r64) <= 1e-3, i
