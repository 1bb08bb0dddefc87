"""Contour files in the reference's layout (contour_writer.f90:193-529): dataset names, shapes,
units and descriptions, the dimensional scaling of every field (data x 1/to_nondim x the unit
system's factor; the sound speed with to_dim = 1), the 32-bit clamp, and the XDMF text."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300.config import SchemeConfig
from fvleg_2d_gb300.contour import _xdmf, contour_datasets
from fvleg_2d_gb300.deck import nondim_factors, parse_deck

DECK = """
[general]
title = 'contour test'
units = 'icf'
[reference_state]
reference_length = 2.0
reference_density = 0.5
reference_velocity = 3.0e5
[time]
max_time = 1
integration_strategy = 'ssp_rk2'
[physics]
polytropic_index = 1.4
[scheme]
flux_solver = 'AUSMPW+'
[initial_conditions]
initial_condition_file = 'x.npz'
"""


def _state(cfg, seed=1):
    r, u, v, p = random_prims(cfg, np.random.default_rng(seed))
    cs = np.sqrt(1.4 * np.abs(p) / np.maximum(r, 1e-30))
    return {"rho": r, "u": u, "v": v, "p": p, "cs": cs}


def test_datasets_scaling_and_shapes():
    deck = parse_deck(DECK)
    f = nondim_factors(deck)
    cfg = SchemeConfig(ni=12, nj=7, dx=0.1, dy=0.2)
    st = _state(cfg)
    xs, ys = np.linspace(0, 1.2, 13), np.linspace(0, 1.4, 8)
    ds = contour_datasets(st, cfg, (xs, ys), 0.25, 1e-3, 42, deck, "t", "icf",
                          plot_volume=True, plot_grid_indices=True)
    g = cfg.ghost_layers()
    inner = lambda a: a[g:-g, g:-g]
    assert ds["iteration"][0] == 42
    assert ds["time"] == (0.25 * 1e9 * (1.0 / f["t_to_nondim"]), "ns", "Simulation Time")
    assert ds["delta_t"][0] == 1e-3 * (1.0 / f["t_to_nondim"]) and ds["delta_t"][1] == "seconds"
    np.testing.assert_array_equal(ds["density"][0],
                                  inner(st["rho"]) * (1.0 / f["density_to_nondim"]) * 1.0)
    np.testing.assert_array_equal(ds["x_velocity"][0],
                                  inner(st["u"]) * (1.0 / f["vel_to_nondim"]) * 1e-5)
    np.testing.assert_array_equal(ds["pressure"][0],
                                  inner(st["p"]) * (1.0 / f["press_to_nondim"]) * 1e-12)
    np.testing.assert_array_equal(ds["sound_speed"][0], inner(st["cs"]) * 1.0 * 1e-5)
    assert ds["pressure"][1] == "Mbar" and ds["x"][1] == "um"
    assert ds["x"][0].shape == (13, 8) and ds["density"][0].shape == (12, 7)
    np.testing.assert_array_equal(ds["x"][0][:, 0], xs * (1.0 / f["len_to_nondim"]) * 1e4)
    np.testing.assert_array_equal(ds["i"][0][:, 0], np.arange(1, 13))
    L = 1.0 / f["len_to_nondim"]
    np.testing.assert_array_equal(ds["volume"][0],
                                  (np.diff(xs)[:, None] * np.diff(ys)[None, :]) * (L * L))


def test_real32_clamp():
    cfg = SchemeConfig(ni=3, nj=2, dx=1.0, dy=1.0)
    st = _state(cfg)
    g = cfg.ghost_layers()
    st["p"][g, g] = 1e300
    st["p"][g + 1, g] = -1e300
    st["p"][g + 2, g] = 1e-300
    ds = contour_datasets(st, cfg, (np.arange(4.0), np.arange(3.0)), 0.0, 0.0, 0,
                          plot_64bit=False)
    p = ds["pressure"][0]
    assert p.dtype == np.float32
    f32 = np.finfo(np.float32)
    assert p[0, 0] == f32.max and p[1, 0] == -f32.max and p[2, 0] == 0.0


def test_xdmf_is_valid_xml():
    text = _xdmf("step_0000042.h5", 12, 7, 0.25, "ns",
                 {"density": "g/cc", "sound_speed": "km/s", "pressure": "Mbar",
                  "x_velocity": "km/s"})
    root = ET.fromstring(text)
    grid = root.find("Domain/Grid")
    assert grid.find("Topology").get("NumberOfElements") == "8 13"
    names = [a.get("Name") for a in grid.findall("Attribute")]
    assert names == ["Density [g/cc]", "Sound Speed [km/s]", "Pressure [Mbar]",
                     "Velocity [km/s]", "Mach"]
    items = [d.text for d in grid.iter("DataItem") if d.text and d.text.strip()]
    assert "step_0000042.h5:/density" in items and "step_0000042.h5:/x" in items


def test_unsupported_format(tmp_path):
    from fvleg_2d_gb300.contour import write_contour

    class F:
        cfg = SchemeConfig(ni=3, nj=2, dx=1.0, dy=1.0)
        iteration, time, last_dt = 0, 0.0, 0.0

        def state(self, names):
            return _state(self.cfg)

    with pytest.raises(ValueError, match="Unsupported"):
        write_contour(F(), str(tmp_path), fmt="vtk")
    paths = write_contour(F(), str(tmp_path), fmt="xdmf")
    assert paths["data"].endswith("step_0000000.h5")
    from fvleg_2d_gb300 import h5lite

    with h5lite.H5File(paths["data"]) as h5:
        assert h5.read("density").shape == (2, 3)  # stored transposed, as HDF5 from Fortran
        assert h5.attrs("density")["units"] == "g/cc"
        assert h5.read("iteration") == 0 and isinstance(h5.read("title"), str)
        assert "step_0000000.h5:/density" in open(paths["xdmf"]).read()
    z = np.load(write_contour(F(), str(tmp_path), fmt="npz")["data"])
    assert z["density"].shape == (2, 3)
    assert str(z["density.units"]) == "g/cc"
