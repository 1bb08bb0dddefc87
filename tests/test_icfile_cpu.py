"""Initial-condition files in pycato's layout (generate_initial_grids.py:603-672) as the
reference reads them (grid_block_2d.f90:216-263, mod_fluid.f90:256-363): shapes, the transposed
storage, ghost-layer check, interior extraction, non-dimensionalization and the rectilinear
check.  The grids are built the way pycato builds them (make_uniform_grid's linspace over the
ghost-extended range, make_2d_layered_grid's stitched layers), restated here."""
import importlib.util

import numpy as np
import pytest

from fvleg_2d_gb300.deck import parse_deck, t_to_nondim
from fvleg_2d_gb300.icfile import ICFileError, read_ic, write_ic


def uniform_nodes(n, lo, hi, ng):
    """make_uniform_grid (generate_initial_grids.py:67-83): linspace over the ghost range."""
    d = float(hi - lo) / float(n)
    return np.linspace(lo - ng * d, hi + ng * d, (n + 1) + 2 * ng, dtype=np.float64)


def layered_nodes(widths_and_counts, ng):
    """Constant-spacing layers stitched with np.unique (generate_initial_grids.py:158-300),
    one ghost node per layer of the outer cell widths on either side."""
    parts, start = [], 0.0
    for thickness, count in widths_and_counts:
        parts.append(np.linspace(start, start + thickness, count + 1))
        start += thickness
    x = np.unique(np.concatenate(parts))
    ldx, rdx = x[1] - x[0], x[-1] - x[-2]
    return np.concatenate([x[0] - ldx * np.arange(ng, 0, -1), x, x[-1] + rdx * np.arange(1, ng + 1)])


def make_file(path, xn, yn, ng, seed=0):
    x2, y2 = np.meshgrid(xn, yn, indexing="ij")
    ni, nj = len(xn) - 1 - 2 * ng, len(yn) - 1 - 2 * ng
    rng = np.random.default_rng(seed)
    shape = (ni + 2 * ng, nj + 2 * ng)
    rho = 1.0 + 0.2 * rng.random(shape)
    u = 1e5 * (rng.random(shape) - 0.5)
    v = 1e5 * (rng.random(shape) - 0.5)
    p = 1e9 * (1.0 + rng.random(shape))
    write_ic(path, x2, y2, rho, u, v, p, ng)
    return (x2, y2, rho, u, v, p), ni, nj


def test_round_trip_and_interior(tmp_path):
    ng = 2
    xn, yn = uniform_nodes(12, 0.0, 1.0, ng), uniform_nodes(7, 0.0, 0.5, ng)
    path = str(tmp_path / "ic.npz")
    (x2, y2, rho, u, v, p), ni, nj = make_file(path, xn, yn, ng)
    z = np.load(path)
    assert z["x"].shape == (nj + 1 + 2 * ng, ni + 1 + 2 * ng)  # stored transposed, as h5py
    assert str(z["density.units"]) == "g/cc"
    ic = read_ic(path, ng, non_dimensionalize=False)
    assert (ic.ni, ic.nj) == (ni, nj)
    np.testing.assert_array_equal(ic.x_nodes, xn[ng:ng + ni + 1])
    np.testing.assert_array_equal(ic.y_nodes, yn[ng:ng + nj + 1])
    for got, want in zip(ic.primitives, (rho, u, v, p)):
        assert got.flags.f_contiguous and got.shape == want.shape
        np.testing.assert_array_equal(got[ng:-ng, ng:-ng], want[ng:-ng, ng:-ng])
        assert not got[:ng].any() and not got[:, -ng:].any()


def test_linspace_grid_widths_vary(tmp_path):
    """pycato's linspace nodes give cell widths that differ in the last bits, so the reference
    computes its metrics per cell: such a file needs the rectilinear grid."""
    ng = 2
    path = str(tmp_path / "ic.npz")
    make_file(path, uniform_nodes(30, 0.0, 1.0, ng), uniform_nodes(10, 0.0, 0.3, ng), ng)
    ic = read_ic(path, ng)
    assert ic.uniform is None
    assert np.ptp(np.diff(ic.x_nodes)) > 0
    path2 = str(tmp_path / "ic2.npz")
    make_file(path2, np.arange(-2, 35) / 32.0, np.arange(-2, 15) / 16.0, ng)
    assert read_ic(path2, ng).uniform == (1 / 32.0, 1 / 16.0)


def test_non_dimensional_scaling(tmp_path):
    ng = 3
    path = str(tmp_path / "ic.npz")
    xn = layered_nodes([(0.1, 10), (0.4, 8), (0.5, 25)], ng)
    (x2, y2, rho, u, v, p), ni, nj = make_file(path, xn, uniform_nodes(6, 0, 0.2, ng), ng)
    L, R, V = 0.25, 2.5, 3.0e5
    ic = read_ic(path, ng, L, R, V)
    np.testing.assert_array_equal(ic.x_nodes, xn[ng:ng + ni + 1] * (1.0 / L))
    np.testing.assert_array_equal(ic.primitives[0][ng:-ng, ng:-ng], rho[ng:-ng, ng:-ng] * (1.0 / R))
    np.testing.assert_array_equal(ic.primitives[1][ng:-ng, ng:-ng], u[ng:-ng, ng:-ng] * (1.0 / V))
    np.testing.assert_array_equal(ic.primitives[3][ng:-ng, ng:-ng],
                                  p[ng:-ng, ng:-ng] * (1.0 / (R * (V * V))))
    deck = parse_deck("[reference_state]\nreference_length = 0.25\nreference_velocity = 3e5\n"
                      "reference_density = 2.5\n[time]\nmax_time = 1\n"
                      "integration_strategy = 'ssp_rk2'\n[physics]\npolytropic_index = 1.4\n"
                      "[scheme]\nflux_solver = 'AUSMPW+'\n"
                      "[initial_conditions]\ninitial_condition_file = 'ic.npz'\n")
    assert t_to_nondim(deck) == 1.0 / (0.25 / 3e5)


def test_errors(tmp_path):
    ng = 2
    path = str(tmp_path / "ic.npz")
    xn, yn = uniform_nodes(8, 0.0, 1.0, ng), uniform_nodes(5, 0.0, 1.0, ng)
    make_file(path, xn, yn, ng)
    with pytest.raises(ICFileError, match="ghost layers"):
        read_ic(path, 3)
    with pytest.raises(ICFileError, match="not found"):
        read_ic(str(tmp_path / "missing.npz"), 2)
    # a sheared (curvilinear) grid
    x2, y2 = np.meshgrid(xn, yn, indexing="ij")
    z = np.zeros((len(xn) - 1, len(yn) - 1))
    write_ic(str(tmp_path / "shear.npz"), x2 + 0.1 * y2, y2, z + 1, z, z, z + 1, ng)
    with pytest.raises(ICFileError, match="not rectilinear"):
        read_ic(str(tmp_path / "shear.npz"), ng)
    if importlib.util.find_spec("h5py") is None:
        (tmp_path / "ic.h5").write_bytes(b"not an HDF5 file")
        with pytest.raises(ICFileError, match="not an HDF5 file"):
            read_ic(str(tmp_path / "ic.h5"), ng)
