"""One grid split into row slabs (fvleg_2d_gb300.slabs), tested with CPU ranks.

Two and three gloo ranks each hold one slab of a grid as an oracle fluid whose cut sides are
exchange sides.  Before every residual evaluation the oracle hands its primitives to the slab
driver's exchange (SlabComm.swap), which fills the ghost rows beyond the cuts with the
neighbours' rows; each step takes the minimum of the slabs' CFL dt.  The slabs must reproduce
the one-grid oracle run bit for bit: state, dt of every step and time.
"""
import json
import os
import socket

import numpy as np
import pytest

from fvleg_2d_gb300 import ic, slabs
from fvleg_2d_gb300.config import SchemeConfig

STEPS = 6
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "reference_unit_vectors.json")))


def _cases():
    """(name, cfg, prims): the quadrant scheme, the Kelvin-Helmholtz scheme (periodic x,
    symmetry y), and MLP5 + SLAU on an all-periodic grid (3 ghost rows; the y cut wraps)."""
    out = []
    cfg, p = ic.riemann_quadrant(40)
    out.append(("quadrant", cfg, p))
    cfg, p = ic.kelvin_helmholtz(32, roe_entropy_fix="harten")
    out.append(("kh", cfg, p))
    rng = np.random.default_rng(4)
    cfg, p = ic.random_circles(36, 30, rng, flux_solver="SLAU", limiter="MLP5",
                               bc={s: "periodic" for s in ("+x", "-x", "+y", "-y")})
    out.append(("circles_periodic", cfg, p))
    return out


def _rows_of(q, g, ni, nj, side):
    """The g interior rows next to `side` of halo-padded fields q: shape (4, g, ni)."""
    j0 = g if side == "-y" else nj  # array index of the first row
    return np.stack([a[g:g + ni, j0:j0 + g].T for a in q])


def _put_ghosts(q, g, ni, nj, side, rows):
    j0 = 0 if side == "-y" else nj + g
    for a, r in zip(q, rows):
        a[g:g + ni, j0:j0 + g] = r.T


def _oracle_slab_run(O, cfg, prims, comm, rank, steps):
    scfg, j0, j1 = slabs.slab_config(cfg, rank, comm.world)
    f = O.OracleFluid(scfg)
    f.set_primitive(*slabs.slab_fields(cfg, prims, j0, j1))
    g = scfg.ghost_layers()

    def exchange(q):
        ex = {rank: {s: _rows_of(q, g, scfg.ni, scfg.nj, s) for s in comm.sides(rank)}}
        im = comm.swap(ex)
        for s, rows in im[rank].items():
            _put_ghosts(q, g, scfg.ni, scfg.nj, s, rows)

    f.set_exchange(exchange)
    dts = []
    for _ in range(steps):
        dt = comm.min([f.get_timestep()])
        ec = comm.code([f.integrate(dt)])
        dts.append(dt)
        assert ec == 0
    st = f.state()
    f.set_exchange(None)
    return {"rho": st["rho"][g:-g, g:-g].tolist(), "rho_E": st["rho_E"][g:-g, g:-g].tolist(),
            "dts": dts, "time": f.time, "j0": j0, "j1": j1}


def _rank_main(rank, world, port, out_path):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import oracle as O
    import torch.distributed as dist

    from fvleg_2d_gb300 import slabs as S

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    res = {}
    for name, cfg, prims in _cases():
        comm = S.SlabComm(world, cfg.bc["+y"] == "periodic", dist=dist)
        res[name] = _oracle_slab_run(O, cfg, prims, comm, rank, STEPS)
    with open(f"{out_path}.{rank}", "w") as fh:
        json.dump(res, fh)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_split_rows_and_slab_configs():
    assert slabs.split_rows(10, 3, 2) == [(0, 4), (4, 7), (7, 10)]
    with pytest.raises(ValueError):
        slabs.split_rows(5, 3, 2)
    cfg, _ = ic.riemann_quadrant(16)
    s0, j0, j1 = slabs.slab_config(cfg, 0, 2)
    s1, k0, k1 = slabs.slab_config(cfg, 1, 2)
    assert (j0, j1, k0, k1) == (0, 8, 8, 16)
    assert s0.bc["+y"] == "exchange" and s0.bc["-y"] == "zero_gradient"
    assert s1.bc["-y"] == "exchange" and s1.bc["+y"] == "zero_gradient"
    assert s0.nj == 8 and s0.bc["+x"] == "zero_gradient"
    per = SchemeConfig(ni=16, nj=16, dx=1 / 16, dy=1 / 16,
                       bc={s: "periodic" for s in ("+x", "-x", "+y", "-y")})
    p0, _, _ = slabs.slab_config(per, 0, 2)
    assert p0.bc["-y"] == p0.bc["+y"] == "exchange" and p0.bc["+x"] == "periodic"
    assert slabs.neighbour(0, "-y", 3, True) == 2 and slabs.neighbour(0, "-y", 3, False) is None
    # the whole grid's order of error checks: NaN, then negative density, then pressure
    assert slabs.first_code([0, 2, 1]) == 1 and slabs.first_code([2, 3]) == 3
    assert slabs.first_code([0, 0]) == 0


def test_local_swap_routes_rows_to_the_neighbours():
    for world, periodic in ((3, False), (3, True), (2, True)):
        comm = slabs.SlabComm(world, periodic)
        ex = {r: {s: np.full((4, 2, 5), 10 * r + (1 if s == "+y" else 0), dtype=float)
                  for s in comm.sides(r)} for r in range(world)}
        im = comm.swap(ex)
        for r in range(world):
            assert sorted(im[r]) == sorted(comm.sides(r))
            for s, rows in im[r].items():
                nb = slabs.neighbour(r, s, world, periodic)
                # beyond my -y side: the neighbour's rows next to its +y side, and vice versa
                assert rows[0, 0, 0] == 10 * nb + (1 if s == "-y" else 0)


def test_exchange_reproduces_the_reference_halo_rows():
    """The reference's own halo-exchange test (tests/unit/test_field/test_field.f90,
    test_halo_exchange: an 8x8 field over 2x2 images, 2 halo cells) asserts the rows each image
    receives across j.  Cut the same field into 2 row slabs (all columns each): the rows the slab
    exchange puts beyond each cut equal the asserted rows on every column they share (the
    columns beyond the x boundary are boundary-condition ghosts there, not exchanged rows)."""
    gold = GOLDEN["field_halo"]
    ni, nj, g = gold["ni"], gold["nj"], gold["n_halo"]
    field = np.zeros((ni + 2 * g, nj + 2 * g), order="F")  # (1-g:ni+g, 1-g:nj+g)
    for img in gold["images"].values():
        for j, row in img["rows"].items():
            field[row["i0"] - 1 + g:row["i1"] + g, int(j) - 1 + g] = row["values"]
    comm = slabs.SlabComm(2, False)
    parts = slabs.split_rows(nj, 2, g)  # rows 1-4 and 5-8: the images' j split
    # four copies of the field stand in for rho, u, v, p
    q = {r: [field[:, j0:j1 + 2 * g].copy(order="F") for _ in range(4)]
         for r, (j0, j1) in enumerate(parts)}
    ex = {r: {s: _rows_of(q[r], g, ni, parts[r][1] - parts[r][0], s) for s in comm.sides(r)}
          for r in q}
    im = comm.swap(ex)
    for r, (j0, j1) in enumerate(parts):
        for s, rows in im[r].items():
            _put_ghosts(q[r], g, ni, j1 - j0, s, rows)
    checked = 0
    for name, img in gold["images"].items():
        k = int(name)
        i_lo = 1 if k in (1, 3) else 5                  # first interior column of the image
        r = 0 if k in (1, 2) else 1                     # the slab holding its rows
        j0, j1 = parts[r]
        for key, want in img["halo_rows"].items():
            jj = {"jhi_halo": j1 + g, "jhi_halo-1": j1 + g - 1,
                  "jlo_halo": j0 + 1 - g, "jlo_halo+1": j0 + 2 - g}[key]  # global 1-based j
            if not (1 <= jj <= nj) or (j0 < jj <= j1):
                continue  # a physical boundary row, or not beyond a cut
            local = jj - (j0 + 1 - g)  # row index in the slab's halo-padded array
            for pos, val in enumerate(want):
                i = i_lo - g + pos  # global 1-based column of the asserted entry
                if 1 <= i <= ni:
                    assert q[r][0][i - 1 + g, local] == val, (name, key, i)
                    checked += 1
    assert checked >= 40


def test_oracle_config_accepts_exchange_on_y_only(oracle):
    cfg, _ = ic.riemann_quadrant(16)
    s0, _, _ = slabs.slab_config(cfg, 0, 2)
    assert oracle.OracleFluid(s0)
    bad = SchemeConfig(ni=16, nj=16, dx=1 / 16, dy=1 / 16,
                       bc={"+x": "exchange", "-x": "zero_gradient", "+y": "zero_gradient",
                           "-y": "zero_gradient"})
    with pytest.raises(ValueError):
        oracle.OracleFluid(bad)


@pytest.mark.parametrize("world", [2, 3])
def test_slabs_over_gloo_ranks_match_the_one_grid_run(oracle, tmp_path, world):
    mp = pytest.importorskip("torch.multiprocessing")
    out = tmp_path / "slabs"
    mp.start_processes(_rank_main, args=(world, _free_port(), str(out)), nprocs=world,
                       join=True, start_method="spawn")
    per_rank = [json.loads((tmp_path / f"slabs.{r}").read_text()) for r in range(world)]
    for name, cfg, prims in _cases():
        ref = oracle.OracleFluid(cfg)
        ref.set_primitive(*prims)
        dts = []
        for _ in range(STEPS):
            dt = ref.get_timestep()
            assert ref.integrate(dt) == 0
            dts.append(dt)
        g = cfg.ghost_layers()
        st = ref.state()
        for r in range(world):
            got = per_rank[r][name]
            assert got["dts"] == dts, (name, r)
            assert got["time"] == ref.time, (name, r)
            j0, j1 = got["j0"], got["j1"]
            for k in ("rho", "rho_E"):
                np.testing.assert_array_equal(np.array(got[k]), st[k][g:-g, g:-g][:, j0:j1],
                                              err_msg=f"{name} slab {r} {k}")
