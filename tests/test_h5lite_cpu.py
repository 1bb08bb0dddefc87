"""The HDF5 reader and writer (fvleg_2d_gb300/h5lite.py), with no HDF5 library.

Known answer: the reference's own HDF5 file, tests/unit/simple.h5, copied byte for byte to
tests/golden/reference_simple.h5 by tests/golden/make_golden.py.  The reference's
make_simple_grid.py wrote it through h5py: a scalar int64 /n_ghost_layers; /x, /y (9 x 9 nodes)
and /density, /x_velocity, /y_velocity, /pressure (8 x 8 cells), transposed, gzip-compressed in
chunks, each with a variable-length string "units" attribute.  Its values are known from the
script: nodes from linspace over [-4, 4] x [-2, 2] with 2 ghost layers, and the four fields equal
to the cartoon rows that tests/golden/reference_unit_vectors.json holds.
"""
import json
import os

import numpy as np
import pytest

from fvleg_2d_gb300 import h5lite
from fvleg_2d_gb300.icfile import read_ic, write_ic

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")
FIXTURE = os.path.join(GOLDEN_DIR, "reference_simple.h5")
GOLDEN = json.load(open(os.path.join(GOLDEN_DIR, "reference_unit_vectors.json")))


def _expected_fields():
    """(i, j) halo-padded field of simple.h5 from the golden rows."""
    sg = GOLDEN["simple_grid"]
    ni, nj, ng = sg["ni"], sg["nj"], sg["n_ghost"]
    data = np.zeros((ni + 2 * ng, nj + 2 * ng))
    for j, row in sg["rows"].items():
        data[ng:ng + ni, int(j) - 1 + ng] = row
    return sg, data


def test_reads_the_reference_simple_h5():
    sg, data = _expected_fields()
    ng = sg["n_ghost"]
    with h5lite.H5File(FIXTURE) as h5:
        assert h5.keys() == ["density", "n_ghost_layers", "pressure", "x", "x_velocity", "y",
                             "y_velocity"]
        assert h5.read("n_ghost_layers") == ng
        units = {"x": "cm", "y": "cm", "density": "g/cc", "x_velocity": "cm/s",
                 "y_velocity": "cm/s", "pressure": "barye"}
        for name, unit in units.items():
            assert h5.attrs(name) == {"units": unit}
        # cells: stored transposed (h5py wrote data.T of the (i, j) array)
        for name in ("density", "x_velocity", "y_velocity", "pressure"):
            a = h5.read(name)
            assert a.dtype == np.float64 and a.shape == data.T.shape
            np.testing.assert_array_equal(a.T, data)
        # nodes: linspace with the ghost nodes, meshgrid(y, x) -> x varies along i
        x0, x1 = sg["xrange"]
        y0, y1 = sg["yrange"]
        dx, dy = (x1 - x0) / sg["ni"], (y1 - y0) / sg["nj"]
        xs = np.linspace(x0 - ng * dx, x1 + ng * dx, sg["ni"] + 1 + 2 * ng)
        ys = np.linspace(y0 - ng * dy, y1 + ng * dy, sg["nj"] + 1 + 2 * ng)
        np.testing.assert_array_equal(h5.read("x").T, np.broadcast_to(xs[:, None],
                                                                     (len(xs), len(ys))))
        np.testing.assert_array_equal(h5.read("y").T, np.broadcast_to(ys[None, :],
                                                                     (len(xs), len(ys))))


def test_read_ic_of_the_reference_file():
    sg, data = _expected_fields()
    ng = sg["n_ghost"]
    ic = read_ic(FIXTURE, ng, non_dimensionalize=False)
    assert (ic.ni, ic.nj) == (sg["ni"], sg["nj"])
    assert ic.uniform == ((sg["xrange"][1] - sg["xrange"][0]) / sg["ni"],
                          (sg["yrange"][1] - sg["yrange"][0]) / sg["nj"])
    for a in ic.primitives:
        np.testing.assert_array_equal(a[ng:-ng, ng:-ng], data[ng:-ng, ng:-ng])


def test_write_read_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    ds = {f"field_{k:02d}": (rng.standard_normal((4 + k, 3)), {"units": "cm",
                                                               "description": f"field {k}"})
          for k in range(12)}
    ds["n_ghost_layers"] = (np.int64(3), {})
    ds["time"] = (np.float64(0.125), {"units": "ns"})
    ds["title"] = ("a run title", {})
    ds["f32"] = (np.linspace(0, 1, 6, dtype=np.float32).reshape(2, 3), {})
    ds["i32"] = (np.arange(5, dtype=np.int32), {"scale": np.float64(0.5)})
    path = str(tmp_path / "t.h5")
    h5lite.write_file(path, ds, root_attrs={"cato_version": "x", "iteration": np.int64(9)})
    raw = open(path, "rb").read()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 0  # superblock version 0
    assert int.from_bytes(raw[40:48], "little") == len(raw)  # end-of-file address
    with h5lite.H5File(path) as h5:
        assert h5.keys() == sorted(ds)
        assert h5.attrs("") == {"cato_version": "x", "iteration": 9}
        for name, (val, attrs) in ds.items():
            got = h5.read(name)
            if isinstance(val, str):
                assert got == val
                continue
            val = np.asarray(val)
            assert np.asarray(got).shape == val.shape and np.asarray(got).dtype == val.dtype
            np.testing.assert_array_equal(got, val)
            assert h5.attrs(name) == attrs


def test_write_ic_h5_round_trip(tmp_path):
    ng, ni, nj = 2, 6, 4
    xs = np.linspace(-ng * 0.5, (ni + ng) * 0.5, ni + 1 + 2 * ng)
    ys = np.linspace(-ng * 0.25, (nj + ng) * 0.25, nj + 1 + 2 * ng)
    x, y = np.meshgrid(xs, ys, indexing="ij")
    rng = np.random.default_rng(8)
    f = [rng.uniform(0.5, 2.0, (ni + 2 * ng, nj + 2 * ng)) for _ in range(4)]
    write_ic(str(tmp_path / "ic.h5"), x, y, *f, ng)
    write_ic(str(tmp_path / "ic.npz"), x, y, *f, ng)
    a = read_ic(str(tmp_path / "ic.h5"), ng)
    b = read_ic(str(tmp_path / "ic.npz"), ng)
    np.testing.assert_array_equal(a.x_nodes, b.x_nodes)
    np.testing.assert_array_equal(a.y_nodes, b.y_nodes)
    for p, q in zip(a.primitives, b.primitives):
        np.testing.assert_array_equal(p, q)


def test_rejects_what_it_cannot_read(tmp_path):
    p = tmp_path / "bad.h5"
    p.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes([2]) + bytes(40))
    with pytest.raises(h5lite.H5Error, match="superblock version 2"):
        h5lite.H5File(str(p))
    with h5lite.H5File(FIXTURE) as h5, pytest.raises(KeyError):
        h5.read("nothing")
