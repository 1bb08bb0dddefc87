"""One grid split into slabs of rows, one slab per GPU (the single-grid configurations on
several GPUs).

The reference decomposes the grid over coarray images: before every residual evaluation,
``time_derivative`` calls ``sync_fields``, which swaps the n_ghost edge rows and columns of rho,
u, v and p with the neighbouring images (``mod_fluid.f90:452-458, 485``;
``field_2d_t%sync_edges``, ``field_2d.f90:551-654``), and the CFL dt is the minimum over the
images (``get_timestep`` -> ``min_to_all``, ``mod_fluid.f90:518-562``,
``mod_collectives.f90:159-163``).

Here the grid is cut along j only.  A slab is an ordinary handle whose cut sides have the
boundary type ``exchange`` (``CATO_BC_EXCHANGE``): its buffers hold n_ghost rows beyond each cut,
and before every RK stage the host copies the neighbours' edge rows of that stage's input into
them (``cato_gpu_halo_export`` / ``cato_gpu_halo_import``).  Each step takes the minimum of the
slabs' CFL dt.  The x boundaries treat the copied rows as interior rows, so every cell sees the
stencil values it sees in the whole grid and the slabs reproduce the one-grid run bit for bit.

:class:`SlabComm` moves the rows: between slabs of one process directly, and between processes
with ``torch.distributed`` point-to-point messages of host buffers (gloo; one slab per rank).
The exchange is host-staged: every stage waits for its neighbours' rows.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .config import SchemeConfig

SIDE_LO, SIDE_HI = "-y", "+y"
_OPPOSITE = {SIDE_LO: SIDE_HI, SIDE_HI: SIDE_LO}
_TAG = {SIDE_LO: 11, SIDE_HI: 12}
# the single grid's order of error checks (the pressure-input target, NaN, negative density,
# negative pressure): each slab reports the first of its own, the grid the first over the slabs
_CODE_ORDER = (17, 3, 1, 2)


def split_rows(nj: int, world: int, ng: int) -> list[tuple[int, int]]:
    """[j0, j1) interior rows (0-based) of each slab: as even as possible, each >= ng rows."""
    if world < 1 or nj < world * ng:
        raise ValueError(f"{nj} rows cannot make {world} slabs of at least {ng} rows")
    base, extra = divmod(nj, world)
    out, j = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((j, j + n))
        j += n
    return out


def slab_config(cfg: SchemeConfig, rank: int, world: int) -> tuple[SchemeConfig, int, int]:
    """The configuration of slab `rank` of `world` and its rows [j0, j1) in the whole grid.
    Inner cuts become ``exchange`` sides; a periodic y axis wraps (the first and the last slab
    exchange with each other).  Rectilinear grids pass the slab's own y nodes to the handle."""
    g = cfg.ghost_layers()
    j0, j1 = split_rows(cfg.nj, world, g)[rank]
    if world == 1:
        return cfg, j0, j1
    bc = dict(cfg.bc)
    periodic_y = bc["+y"] == "periodic"
    if rank > 0 or periodic_y:
        bc["-y"] = "exchange"
    if rank < world - 1 or periodic_y:
        bc["+y"] = "exchange"
    return dataclasses.replace(cfg, nj=j1 - j0, bc=bc), j0, j1


def slab_fields(cfg: SchemeConfig, fields, j0: int, j1: int) -> list[np.ndarray]:
    """Halo-padded slab arrays (rows j0 - g .. j1 + g - 1 with their ghost columns) cut from
    halo-padded arrays of the whole grid.  A slab's ghost rows beyond a cut are the
    neighbours' interior rows; beyond a physical side they are the whole grid's ghosts."""
    g = cfg.ghost_layers()
    return [np.asfortranarray(np.asarray(a)[:, j0:j1 + 2 * g]) for a in fields]


def neighbour(rank: int, side: str, world: int, periodic_y: bool) -> int | None:
    """The slab beyond `side` of slab `rank`, or None at a physical boundary."""
    nb = rank - 1 if side == SIDE_LO else rank + 1
    if 0 <= nb < world:
        return nb
    return nb % world if periodic_y and world > 1 else None


def first_code(codes) -> int:
    """The error code of the whole grid from the slabs' codes (the single grid's check order)."""
    for c in _CODE_ORDER:
        if c in codes:
            return c
    return max(codes) if codes else 0


class SlabComm:
    """Moves edge rows between the slabs of one grid.

    ``local`` lists the slab indices this process holds.  With ``dist`` None every slab is local
    (several handles in one process, e.g. one per GPU from one host thread); otherwise this
    process is slab ``dist.get_rank()`` of ``dist.get_world_size()`` and rows to other slabs go
    as gloo messages."""

    def __init__(self, world: int, periodic_y: bool, local=None, dist=None):
        self.world = world
        self.periodic_y = periodic_y
        self.dist = dist
        if dist is not None:
            if dist.get_world_size() != world:
                raise ValueError("one slab per rank: world size != number of slabs")
            local = [dist.get_rank()]
        self.local = list(range(world)) if local is None else list(local)

    def sides(self, rank: int) -> list[str]:
        return [s for s in (SIDE_LO, SIDE_HI)
                if neighbour(rank, s, self.world, self.periodic_y) is not None]

    def swap(self, exports: dict) -> dict:
        """exports[rank][side] = the n_ghost edge rows next to `side` of local slab `rank`;
        returns imports[rank][side] = the rows that go beyond `side` (the neighbour's rows next
        to its opposite side)."""
        imports = {r: {} for r in self.local}
        pending = []
        if self.dist is not None:
            import torch
        for r in self.local:
            for side in self.sides(r):
                nb = neighbour(r, side, self.world, self.periodic_y)
                rows = exports[r][side]
                if nb in imports:
                    imports[nb][_OPPOSITE[side]] = rows
                    continue
                pending.append(self.dist.isend(torch.from_numpy(np.ascontiguousarray(rows)),
                                               dst=nb, tag=_TAG[side]))
                buf = torch.empty(rows.shape, dtype=torch.float64)
                # my rows beyond `side` are the neighbour's rows next to its opposite side
                pending.append(self.dist.irecv(buf, src=nb, tag=_TAG[_OPPOSITE[side]]))
                imports[r][side] = buf
        for p in pending:
            p.wait()
        for r in imports:
            for side, v in imports[r].items():
                if not isinstance(v, np.ndarray):
                    imports[r][side] = v.numpy()
        return imports

    def _allgather(self, values: list[float]) -> list[float]:
        if self.dist is None:
            return list(values)
        import torch

        t = torch.tensor(values, dtype=torch.float64)
        out = [torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(out, t)
        return [float(x) for o in out for x in o.tolist()]

    def min(self, values: list[float]) -> float:
        """The minimum over every slab (values: one per local slab)."""
        return min(self._allgather(values))

    def code(self, codes: list[int]) -> int:
        return first_code([int(c) for c in self._allgather([float(c) for c in codes])])


class SlabRun:
    """Steps the local slabs (``fluid.Fluid`` handles with exchange sides, one per GPU) of one
    grid together: the minimum CFL dt, then stage by stage with the edge rows swapped before
    each stage.  ``fluids[i]`` is slab ``comm.local[i]``."""

    def __init__(self, fluids, comm: SlabComm):
        if len(fluids) != len(comm.local):
            raise ValueError("one fluid per local slab")
        self.fluids = list(fluids)
        self.comm = comm
        self.stages = fluids[0].stage_count()

    def _swap(self) -> None:
        ex = {r: {s: f.halo_export(s) for s in self.comm.sides(r)}
              for r, f in zip(self.comm.local, self.fluids)}
        im = self.comm.swap(ex)
        for r, f in zip(self.comm.local, self.fluids):
            for s, rows in im[r].items():
                f.halo_import(s, rows)

    def step(self) -> tuple[float, int]:
        """One step of the whole grid: (dt, error code of the whole grid)."""
        dt = self.comm.min([f.get_timestep() for f in self.fluids])
        for f in self.fluids:
            f.step_begin(dt)
        for _ in range(self.stages):
            self._swap()
            for f in self.fluids:
                f.step_stage()
        res = [f.step_end() for f in self.fluids]
        return res[0][0], self.comm.code([ec for _, ec in res])

    def run(self, n_steps: int) -> tuple[int, int]:
        """Up to n_steps steps; stops at the first error.  Returns (steps taken, error code)."""
        for n in range(n_steps):
            _, ec = self.step()
            if ec:
                return n + 1, ec
        return n_steps, 0
