"""Contour files in the reference's layout (``contour_writer_t``,
``src/lib/io/contour_writer.f90:120-529``).

One call writes ``step_<iteration, 7 digits>`` in ``results_dir``: the datasets of
``write_hdf5`` (``:193-384``) -- ``/title``, ``/iteration``, ``/time``, ``/delta_t``,
``/n_ghost_layers``, ``/x``, ``/y`` (interior nodes), ``/density``, ``/x_velocity``,
``/y_velocity``, ``/pressure``, ``/sound_speed``, optionally ``/volume``, ``/i``, ``/j`` -- each
with its ``units`` and ``description`` attributes, dimensional and in the deck's output unit
system (``units.f90:94-143``); and for the ``xdmf`` format the XDMF description of
``write_xdmf`` (``:386-529``) that points at ``<name>.h5:/<dataset>``.

The datasets are written to ``<name>.h5``: with h5py when it is installed, else with
:mod:`fvleg_2d_gb300.h5lite` (superblock version 0, contiguous datasets, fixed-length string
attributes), arrays stored transposed as an HDF5 file written from Fortran reads in C order.
``fmt="npz"`` writes ``<name>.npz`` with the same names, shapes and attributes
(``<dataset>.units``, ``<dataset>.description``) instead.  Scaling follows the reference: a field is written as
``data * to_dim * unit_factor`` with ``to_dim = 1 / to_nondim`` of that field
(``field_2d.f90:490-521, 804-823``); the sound speed is never made non-dimensional there, so it
is written with ``to_dim = 1``; 32-bit output clamps to +-huge(real32) and flushes below
tiny(real32) (``write_2d_real_data``, ``:545-584``).
"""
from __future__ import annotations

import os

import numpy as np

from .deck import nondim_factors

# io_*_units and io_*_label of set_output_unit_system (units.f90:94-143)
UNIT_SYSTEMS = {
    "cgs": {"velocity": (1.0, "cm/s"), "time": (1.0, "s"), "length": (1.0, "cm"),
            "pressure": (1.0, "barye"), "density": (1.0, "g/cc"), "volume": (1.0, "cc")},
    "icf": {"velocity": (1e-5, "km/s"), "time": (1e9, "ns"), "length": (1e4, "um"),
            "pressure": (1e-12, "Mbar"), "density": (1.0, "g/cc"), "volume": (1.0, "cc")},
}

_F32_HUGE = float(np.finfo(np.float32).max)
_F32_TINY = float(np.finfo(np.float32).tiny)


def _to_real32(a: np.ndarray) -> np.ndarray:
    out = np.clip(a, -_F32_HUGE, _F32_HUGE).astype(np.float32)
    out[np.abs(a) < _F32_TINY] = 0.0
    return out


def _uniform_nodes(n: int, d: float) -> np.ndarray:
    return np.arange(n + 1, dtype=np.float64) * d


def contour_datasets(state: dict, cfg, nodes, time: float, delta_t: float, iteration: int,
                     deck=None, title: str = "", unit_system: str = "cgs",
                     plot_64bit: bool = True, plot_volume: bool = False,
                     plot_grid_indices: bool = False) -> dict:
    """The datasets of one contour file as {name: (array or scalar, units, description)}, in
    Fortran (i, j) orientation.  ``state`` holds interior or halo-padded rho, u, v, p, cs."""
    f = nondim_factors(deck) if deck is not None else dict.fromkeys(
        ("len_to_nondim", "t_to_nondim", "density_to_nondim", "density_to_dim",
         "vel_to_nondim", "press_to_nondim"), 1.0)
    us = UNIT_SYSTEMS[unit_system]
    g = cfg.ghost_layers()
    ni, nj = cfg.ni, cfg.nj

    def interior(a):
        a = np.asarray(a, dtype=np.float64)
        return a[g:g + ni, g:g + nj] if a.shape == cfg.halo_shape else a

    t_to_dim = 1.0 / f["t_to_nondim"]
    len_to_dim = 1.0 / f["len_to_nondim"]
    xs, ys = nodes
    x2, y2 = np.meshgrid(np.asarray(xs, np.float64), np.asarray(ys, np.float64), indexing="ij")
    real = (lambda a: a) if plot_64bit else _to_real32
    out = {
        "title": (title, None, None),
        "iteration": (np.int32(iteration), "dimensionless", "Iteration Count"),
        "time": (time * us["time"][0] * t_to_dim, us["time"][1], "Simulation Time"),
        "delta_t": (delta_t * t_to_dim, "seconds", "Simulation Timestep"),
        "n_ghost_layers": (np.int32(g), None, None),
        "x": (real(x2 * len_to_dim * us["length"][0]), us["length"][1], "X Coordinate"),
        "y": (real(y2 * len_to_dim * us["length"][0]), us["length"][1], "Y Coordinate"),
    }
    if plot_grid_indices:
        ii, jj = np.meshgrid(np.arange(1, ni + 1), np.arange(1, nj + 1), indexing="ij")
        out["i"] = (ii.astype(np.int32), "dimensionless", "Cell i Index")
        out["j"] = (jj.astype(np.int32), "dimensionless", "Cell j Index")
    fields = (("density", "rho", 1.0 / f["density_to_nondim"], "density", "Cell Density"),
              ("x_velocity", "u", 1.0 / f["vel_to_nondim"], "velocity", "Cell X Velocity"),
              ("y_velocity", "v", 1.0 / f["vel_to_nondim"], "velocity", "Cell Y Velocity"),
              ("pressure", "p", 1.0 / f["press_to_nondim"], "pressure", "Cell Pressure"),
              ("sound_speed", "cs", 1.0, "velocity", "Cell Sound Speed"))
    for name, key, to_dim, kind, desc in fields:
        out[name] = (real(interior(state[key]) * to_dim * us[kind][0]), us[kind][1], desc)
    if plot_volume:
        w, h = np.diff(xs), np.diff(ys)
        vol = w[:, None] * h[None, :] - 0.0 * 0.0
        out["volume"] = (real(vol * (len_to_dim * len_to_dim) * us["volume"][0]),
                         us["volume"][1], "Cell Volume")
    return out


def _xdmf(h5name: str, ni: int, nj: int, time_value: float, time_label: str, labels: dict) -> str:
    """write_xdmf (contour_writer.f90:386-529) for the datasets of `h5name`."""
    cell = f"{nj} {ni}"
    node = f"{nj + 1} {ni + 1}"

    def item(ds, indent="        "):
        return (f'{indent}<DataItem Dimensions="{cell}" Format="HDF" '
                f'NumberType="Float" Precision="4">{h5name}:/{ds}</DataItem>')

    lines = ['<?xml version="1.0" ?>', '<Xdmf version="2.2">', '  <Domain>',
             '    <Grid GridType="Uniform" Name="grid">',
             f'      <Time Value="{time_value:.3g} {time_label}"/>',
             f'      <Topology NumberOfElements="{node}" TopologyType="2DSMesh"/>',
             '      <Geometry GeometryType="X_Y">']
    for ds in ("x", "y"):
        lines.append(f'        <DataItem Dimensions="{node}" Format="HDF" NumberType="Float" '
                     f'Precision="4">{h5name}:/{ds}</DataItem>')
    lines.append('      </Geometry>')
    for ds, name in (("density", "Density"), ("sound_speed", "Sound Speed"),
                     ("pressure", "Pressure")):
        lines += [f'      <Attribute AttributeType="Scalar" Center="Cell" '
                  f'Name="{name} [{labels[ds]}]">', item(ds), '      </Attribute>']
    lines += [f'      <Attribute AttributeType="Vector" Center="Cell" '
              f'Name="Velocity [{labels["x_velocity"]}]" Dimensions="{cell} 2">',
              f'        <DataItem Dimensions="{cell} 2" ItemType="Function" '
              'Function="JOIN($0, $1)">',
              f'          <DataItem DataType="Float" Dimensions="{cell}" Format="HDF" '
              f'Precision="4">{h5name}:/x_velocity</DataItem>',
              f'          <DataItem DataType="Float" Dimensions="{cell}" Format="HDF" '
              f'Precision="4">{h5name}:/y_velocity</DataItem>',
              '        </DataItem>', '      </Attribute>',
              f'      <Attribute AttributeType="Vector" Center="Cell" Name="Mach" '
              f'Dimensions="{cell} 2">',
              f'        <DataItem Dimensions="{cell} 2" ItemType="Function" '
              'Function="JOIN(ABS($0/$2), ABS($1/$2))">',
              f'          <DataItem DataType="Float" Dimensions="{cell}" Format="HDF" '
              f'Precision="4">{h5name}:/x_velocity</DataItem>',
              f'          <DataItem DataType="Float" Dimensions="{cell}" Format="HDF" '
              f'Precision="4">{h5name}:/y_velocity</DataItem>',
              f'          <DataItem DataType="Float" Dimensions="{cell}" Format="HDF" '
              f'Precision="4">{h5name}:/sound_speed</DataItem>',
              '        </DataItem>', '      </Attribute>',
              '    </Grid>', '  </Domain>', '</Xdmf>']
    return "\n".join(lines) + "\n"


def write_contour(fluid, results_dir: str, deck=None, *, iteration: int | None = None,
                  title: str | None = None, unit_system: str | None = None,
                  fmt: str | None = None, plot_64bit: bool = True, plot_volume: bool = False,
                  plot_grid_indices: bool = False) -> dict:
    """contour_writer_t%write_contour for a Fluid: downloads its state and writes
    ``step_NNNNNNN.{h5|npz}`` (+ ``.xdmf``).  Returns the written paths."""
    st = fluid.state(("rho", "u", "v", "p", "cs"))
    cfg = fluid.cfg
    nodes = getattr(fluid, "nodes", None) or (_uniform_nodes(cfg.ni, cfg.dx),
                                              _uniform_nodes(cfg.nj, cfg.dy))
    it = fluid.iteration if iteration is None else iteration
    t = fluid.time
    dt = fluid.last_dt
    title = title if title is not None else (deck.title if deck is not None else "")
    unit_system = unit_system or (deck.units if deck is not None else "cgs")
    fmt = fmt or (deck.contour_format if deck is not None else "xdmf")
    if fmt not in ("xdmf", "hdf5", "h5", "npz"):
        raise ValueError(f"Unsupported I/O contour format '{fmt}' (must be .xdmf .h5 or .hdf5)")
    ds = contour_datasets(st, cfg, nodes, t, dt, it, deck, title, unit_system, plot_64bit,
                          plot_volume, plot_grid_indices)
    os.makedirs(results_dir, exist_ok=True)
    stem = f"step_{it:07d}"
    paths = {}
    try:
        import h5py
    except ImportError:
        h5py = None
    if fmt != "npz" and h5py is not None:
        path = os.path.join(results_dir, stem + ".h5")
        with h5py.File(path, "w") as h5:
            for name, (val, units, desc) in ds.items():
                d = h5.create_dataset("/" + name, data=val.T if np.ndim(val) == 2 else val)
                if units is not None:
                    d.attrs["units"] = units
                if desc is not None:
                    d.attrs["description"] = desc
    elif fmt != "npz":
        from . import h5lite

        path = os.path.join(results_dir, stem + ".h5")
        out = {}
        for name, (val, units, desc) in ds.items():
            attrs = {k: v for k, v in (("units", units), ("description", desc)) if v is not None}
            out[name] = (val.T if np.ndim(val) == 2 else val, attrs)
        h5lite.write_file(path, out)
    else:
        path = os.path.join(results_dir, stem + ".npz")
        out = {}
        for name, (val, units, desc) in ds.items():
            out[name] = val.T.copy() if np.ndim(val) == 2 else np.asarray(val)
            if units is not None:
                out[name + ".units"] = units
            if desc is not None:
                out[name + ".description"] = desc
        with open(path, "wb") as fh:
            np.savez(fh, **out)
    paths["data"] = path
    if fmt == "xdmf":
        us = UNIT_SYSTEMS[unit_system]
        labels = {k: ds[k][1] for k in ("density", "sound_speed", "pressure", "x_velocity")}
        xpath = os.path.join(results_dir, stem + ".xdmf")
        with open(xpath, "w") as fh:
            fh.write(_xdmf(stem + ".h5", cfg.ni, cfg.nj, ds["time"][0], us["time"][1], labels))
        paths["xdmf"] = xpath
    return paths
