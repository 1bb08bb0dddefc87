"""Initial-condition files in pycato's layout (``pycato/generate_initial_grids.py:603-672``).

The reference reads its grid and initial state from one HDF5 file
(``grid_block_2d_t%read_from_h5``, ``src/lib/grid/grid_block_2d.f90:216-263``, and
``fluid_t%initialize_from_hdf5``, ``src/lib/fluid/mod_fluid.f90:256-363``):

* ``/n_ghost_layers``: must equal the ghost layers the limiter needs;
* ``/x``, ``/y``: node coordinates including the ghost nodes, ``(ni+1+2g) x (nj+1+2g)`` in the
  Fortran (i, j) order (pycato writes the numpy (i, j) array transposed, so a C reader sees
  (j, i)); units ``cm``;
* ``/density``, ``/x_velocity``, ``/y_velocity``, ``/pressure``: cell values including ghosts,
  ``(ni+2g) x (nj+2g)``, same transposition; units ``g/cc``, ``cm/s``, ``barye``.

Only the interior cells and nodes are used.  The reference then scales them to its
non-dimensional units: nodes by ``len_to_nondim`` (``grid_block_2d.f90:260-262``) and the
primitives by ``density_to_nondim``, ``vel_to_nondim`` and ``press_to_nondim``
(``mod_fluid.f90:347-350``; the factors of ``set_refrence_quantities``,
``src/lib/non_dimensional.f90:95-135``).

``.h5`` / ``.hdf5`` files are read through h5py when it is installed, else through
:mod:`fvleg_2d_gb300.h5lite` (the format subset pycato's h5py files use: gzip-compressed chunks,
variable-length string attributes; checked on the reference's own ``tests/unit/simple.h5``).
:func:`write_ic` writes HDF5 the same way (contiguous datasets) for a ``.h5`` / ``.hdf5`` path,
and otherwise an ``.npz`` file with the same dataset names, shapes and transposition (the units
as ``<name>.units`` strings).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

_FIELDS = (("density", "g/cc"), ("x_velocity", "cm/s"), ("y_velocity", "cm/s"),
           ("pressure", "barye"))


class ICFileError(ValueError):
    """An unusable initial-condition file (the reference stops with error_msg)."""


@dataclass
class InitialCondition:
    ni: int
    nj: int
    n_ghost: int
    x_nodes: np.ndarray   # interior nodes x(1..ni+1), non-dimensional
    y_nodes: np.ndarray   # interior nodes y(1..nj+1), non-dimensional
    primitives: list      # rho, u, v, p: halo-padded Fortran-order float64, ghosts 0
    uniform: tuple | None  # (dx, dy) when every cell has the same width and height, else None

    def scheme_grid(self) -> tuple[int, int, float, float]:
        """(ni, nj, dx, dy) for :class:`SchemeConfig`; dx, dy are the first cell's when the
        widths vary (the per-cell widths then come from :meth:`apply_grid`)."""
        dx = float(self.x_nodes[1] - self.x_nodes[0])
        dy = float(self.y_nodes[1] - self.y_nodes[0])
        return self.ni, self.nj, dx, dy

    def apply_grid(self, handle) -> None:
        """Give a Fluid/FluxSolver this file's grid: nothing more for equal cells (their
        metrics are the configuration's dx x dy), else the rectilinear node arrays."""
        if self.uniform is None:
            handle.set_rectilinear(self.x_nodes, self.y_nodes)


def write_ic(path: str, x, y, rho, u, v, p, n_ghost: int) -> None:
    """Write the pycato layout to ``path`` (HDF5 for ``.h5`` / ``.hdf5``, else ``.npz``).
    ``x``, ``y``: node coordinates including ghost nodes, shape (ni+1+2g, nj+1+2g); fields:
    (ni+2g, nj+2g); all in (i, j) order and in cgs units."""
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    if path.endswith((".h5", ".hdf5")):
        from . import h5lite

        ds = {"n_ghost_layers": (np.int64(n_ghost), {}),
              "x": (x.T, {"units": "cm"}), "y": (y.T, {"units": "cm"})}
        for (name, unit), a in zip(_FIELDS, (rho, u, v, p)):
            ds[name] = (np.asarray(a, np.float64).T, {"units": unit})
        h5lite.write_file(path, ds)
        return
    out = {"n_ghost_layers": np.int32(n_ghost), "x": x.T.copy(), "y": y.T.copy(),
           "x.units": "cm", "y.units": "cm"}
    for (name, unit), a in zip(_FIELDS, (rho, u, v, p)):
        out[name] = np.asarray(a, np.float64).T.copy()
        out[name + ".units"] = unit
    with open(path, "wb") as f:
        np.savez(f, **out)


def _load(path: str) -> dict:
    if not os.path.exists(path):
        raise ICFileError(f'File not found: "{path}"')
    if path.endswith((".h5", ".hdf5")):
        names = ("x", "y") + tuple(n for n, _ in _FIELDS)
        try:
            import h5py
        except ImportError:
            h5py = None
        if h5py is not None:
            with h5py.File(path, "r") as h5:
                d = {"n_ghost_layers": np.asarray(h5["/n_ghost_layers"])}
                for name in names:
                    d[name] = np.asarray(h5["/" + name], dtype=np.float64)
                    u = h5["/" + name].attrs.get("units", "")
                    d[name + ".units"] = u.decode() if isinstance(u, bytes) else str(u)
            return d
        from . import h5lite

        try:
            with h5lite.H5File(path) as h5:
                d = {"n_ghost_layers": np.asarray(h5.read("n_ghost_layers"))}
                for name in names:
                    d[name] = np.asarray(h5.read(name), dtype=np.float64)
                    d[name + ".units"] = str(h5.attrs(name).get("units", ""))
        except KeyError as exc:
            raise ICFileError(f"{path}: dataset {exc} missing") from exc
        except h5lite.H5Error as exc:
            raise ICFileError(f"{path}: {exc}") from exc
        return d
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def read_ic(path: str, n_ghost_required: int, reference_length: float = 1.0,
            reference_density: float = 1.0, reference_velocity: float = 1.0,
            non_dimensionalize: bool = True) -> InitialCondition:
    """Read an initial-condition file, check it against the scheme's ghost layers and return
    its interior grid and primitives in the reference's non-dimensional units."""
    d = _load(path)
    ng = int(np.asarray(d["n_ghost_layers"]).reshape(-1)[0])
    if ng != n_ghost_required:
        raise ICFileError(f"The number of ghost layers in the file ({ng}) does not match the "
                          f"input requirement set by the edge interpolation scheme "
                          f"({n_ghost_required})")
    x, y = d["x"].T, d["y"].T  # back to (i, j)
    if x.shape != y.shape or x.ndim != 2:
        raise ICFileError(f"/x {x.shape} and /y {y.shape} must be 2-D arrays of one shape")
    ni, nj = x.shape[0] - 1 - 2 * ng, x.shape[1] - 1 - 2 * ng
    if ni < 1 or nj < 1:
        raise ICFileError(f"grid of {x.shape} nodes has no interior cells with {ng} ghost layers")
    for name, _ in _FIELDS:
        if d[name].T.shape != (ni + 2 * ng, nj + 2 * ng):
            raise ICFileError(f"/{name} has shape {d[name].T.shape}, expected "
                              f"{(ni + 2 * ng, nj + 2 * ng)}")
    xi = x[ng:ng + ni + 1, ng:ng + nj + 1]
    yi = y[ng:ng + ni + 1, ng:ng + nj + 1]
    # every pycato grid is a meshgrid of one x and one y array; the kernels need exactly that
    if not (np.all(xi == xi[:, :1]) and np.all(yi == yi[:1, :])):
        raise ICFileError("the grid is not rectilinear (x must depend on i only and y on j "
                          "only); curvilinear grids are not supported")
    if non_dimensionalize:
        vel_ref = reference_velocity
        len_to_nondim = 1.0 / reference_length
        density_to_nondim = 1.0 / reference_density
        vel_to_nondim = 1.0 / vel_ref
        press_to_nondim = 1.0 / (reference_density * (vel_ref * vel_ref))
    else:
        len_to_nondim = density_to_nondim = vel_to_nondim = press_to_nondim = 1.0
    xs = np.ascontiguousarray(xi[:, 0]) * len_to_nondim
    ys = np.ascontiguousarray(yi[0, :]) * len_to_nondim
    if not (np.all(np.diff(xs) > 0) and np.all(np.diff(ys) > 0)):
        raise ICFileError("node coordinates must be strictly increasing")
    prims = []
    for (name, _), fac in zip(_FIELDS, (density_to_nondim, vel_to_nondim, vel_to_nondim,
                                        press_to_nondim)):
        a = np.zeros((ni + 2 * ng, nj + 2 * ng), dtype=np.float64, order="F")
        a[ng:ng + ni, ng:ng + nj] = d[name].T[ng:ng + ni, ng:ng + nj] * fac
        prims.append(a)
    wx, wy = np.diff(xs), np.diff(ys)
    uniform = (float(wx[0]), float(wy[0])) if (np.all(wx == wx[0]) and
                                               np.all(wy == wy[0])) else None
    return InitialCondition(ni, nj, ng, xs, ys, prims, uniform)
