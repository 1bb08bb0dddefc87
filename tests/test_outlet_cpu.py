"""The oracle's outlet boundary condition against a direct transcription of
outlet_bc.f90:83-175 in numpy (the reference's tests do not exercise the outlet), and the
configuration rules both sides share."""
import ctypes

import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300 import _lib
from fvleg_2d_gb300.config import SchemeConfig

TINY = np.finfo(np.float64).tiny


def _outlet_px(cfg, rho, u, v, p, gamma, p_b):
    """+x ghost columns from the boundary column ihi, for every j of the halo."""
    g = cfg.ghost_layers()
    ihi = g + cfg.ni - 1
    for i in range(ihi + 1, ihi + 1 + g):
        for j in range(rho.shape[1]):
            p_d, rho_0 = p[ihi, j], rho[ihi, j]
            if p_b > TINY and rho_0 > TINY:
                cs = np.sqrt(gamma * abs(p_d / rho_0))
                vel = np.sqrt(u[ihi, j] * u[ihi, j] + v[ihi, j] * v[ihi, j])
                mach = vel / cs
                nx = u[ihi, j] / (vel + 1e-30)
                ny = v[ihi, j] / (vel + 1e-30)
                if mach > 1.0:
                    rho[i, j], u[i, j], v[i, j], p[i, j] = rho[ihi, j], u[ihi, j], v[ihi, j], p[ihi, j]
                else:
                    rho[i, j] = rho[ihi, j] + (p_b - p_d) / (cs * cs)
                    u[i, j] = u[ihi, j] + nx * (p_d - p_b) / (rho_0 * cs)
                    v[i, j] = v[ihi, j] + ny * (p_d - p_b) / (rho_0 * cs)
                    p[i, j] = p_b


def test_oracle_outlet_matches_transcription(oracle):
    bc = {"+x": "outflow", "-x": "outflow", "+y": "zero_gradient", "-y": "symmetry"}
    cfg = SchemeConfig(ni=12, nj=9, dx=0.1, dy=0.1, bc=bc, gamma=1.4,
                       outflow_ambient_pressure=0.8)
    prims = random_prims(cfg, np.random.default_rng(2))
    g = cfg.ghost_layers()
    prims[1][g:-g, g:-g] *= 3.0
    got = [a.copy(order="F") for a in prims]
    oracle.apply_bc(cfg, *got)
    ref = [a.copy(order="F") for a in prims]
    r, u, v, p = ref
    # priority 1 first (+y zero gradient, then -y symmetry: full rows), then priority 0 outlets
    # in +x, -x order (+x: characteristic; -x: full-column copy)
    for gg in range(1, g + 1):
        for a in ref:
            a[:, g + cfg.nj - 1 + gg] = a[:, g + cfg.nj - 1]
    for gg in range(1, g + 1):
        for k, a in enumerate(ref):
            a[:, g - gg] = -a[:, g + gg - 1] if k == 2 else a[:, g + gg - 1]
    _outlet_px(cfg, r, u, v, p, 1.4, 0.8)
    for gg in range(1, g + 1):
        for a in ref:
            a[g - gg, :] = a[g, :]
    for k in range(4):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=f"var {k}")


@pytest.mark.parametrize("p_b,ok", [(0.5, True), (0.0, False), (-1.0, False)])
def test_outlet_needs_positive_pressure(oracle, p_b, ok):
    bc = {"+x": "outflow", "-x": "zero_gradient", "+y": "zero_gradient", "-y": "zero_gradient"}
    c = SchemeConfig(ni=8, nj=8, dx=0.1, dy=0.1, bc=bc, gamma=1.4,
                     outflow_ambient_pressure=p_b).to_c()
    L = _lib.load(build_if_missing=True)
    assert (L.cato_config_check(ctypes.byref(c)) == 0) == ok
    assert (oracle.lib().oracle_config_check(ctypes.byref(c)) == 0) == ok
