"""Shared test setup: import paths, the `gpu` marker, oracle and library fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def cato_lib():
    """The product library; GPU tests fail loudly when it is missing (no CPU fallback)."""
    from fvleg_2d_gb300 import _lib

    return _lib.load(build_if_missing=True)


def random_prims(cfg, rng, jumps=True):
    """Positive density/pressure fields with smooth variation plus a few discontinuities,
    interior only (ghosts 0), halo-padded Fortran order."""
    g = cfg.ghost_layers()
    ni, nj = cfg.ni, cfg.nj
    x = (np.arange(ni) + 0.5)[:, None] / ni
    y = (np.arange(nj) + 0.5)[None, :] / nj
    out = []
    for k in range(4):
        base = np.sin(2 * np.pi * (x * (k + 1) + 0.3 * y)) * np.cos(2 * np.pi * y * (k + 2))
        noise = rng.normal(0.0, 0.05, (ni, nj))
        f = base + noise
        if jumps:
            f = f + 0.8 * (x > 0.37 + 0.2 * y) - 0.5 * ((x - 0.6) ** 2 + (y - 0.4) ** 2 < 0.04)
        if k in (0, 3):  # density, pressure > 0
            f = 1.0 + 0.45 * f / np.abs(f).max()
            f = np.maximum(f, 0.05)
        else:
            f = 0.6 * f
        a = np.zeros(cfg.halo_shape, order="F")
        a[g:g + ni, g:g + nj] = f
        out.append(a)
    return out


def interior(cfg, a):
    g = cfg.ghost_layers()
    return a[g:g + cfg.ni, g:g + cfg.nj]
