"""One grid split into row slabs on the GPU, through the C-ABI's stage-by-stage step and halo
export/import (fvleg_2d_gb300.slabs).

The slabs are handles of one process on one GPU, stepped together by SlabRun with the edge rows
copied through the host before every stage (the exchange a multi-GPU run makes between
processes); no kernel waits for another.  The slabs must give the one-grid run bit for bit in
every precision: the dt of every step, the time and the state.
"""
import dataclasses

import numpy as np
import pytest

from fvleg_2d_gb300 import ic, slabs
from fvleg_2d_gb300.fluid import CatoError, Fluid
from fvleg_2d_gb300.batch import Batch

pytestmark = pytest.mark.gpu

STEPS = 8


def _case(name, precision):
    if name == "quadrant":
        return ic.riemann_quadrant(64, precision=precision)
    if name == "kh":
        return ic.kelvin_helmholtz(64, roe_entropy_fix="harten", precision=precision)
    rng = np.random.default_rng(4)
    return ic.random_circles(48, 40, rng, flux_solver="SLAU", limiter="MLP5", precision=precision,
                             bc={s: "periodic" for s in ("+x", "-x", "+y", "-y")})


@pytest.mark.parametrize("precision", ["fp64", "mixed_df", "mixed"])
@pytest.mark.parametrize("name,world", [("quadrant", 2), ("quadrant", 3), ("kh", 2),
                                        ("circles_periodic", 2), ("circles_periodic", 3)])
def test_slabs_match_the_one_grid_run(cato_lib, name, world, precision):
    cfg, prims = _case(name, precision)
    one = Fluid(cfg).initialize(*prims)
    dts = []
    for _ in range(STEPS):
        dt, ec = one.integrate()
        assert ec == 0
        dts.append(dt)
    comm = slabs.SlabComm(world, cfg.bc["+y"] == "periodic")
    parts = [slabs.slab_config(cfg, r, world) for r in range(world)]
    fluids = [Fluid(c).initialize(*slabs.slab_fields(cfg, prims, j0, j1)) for c, j0, j1 in parts]
    run = slabs.SlabRun(fluids, comm)
    got = []
    for _ in range(STEPS):
        dt, ec = run.step()
        assert ec == 0
        got.append(dt)
    assert got == dts
    g = cfg.ghost_layers()
    ref = one.state(("rho", "rho_u", "rho_v", "rho_E"))
    for f, (c, j0, j1) in zip(fluids, parts):
        assert f.time == one.time
        st = f.state(("rho", "rho_u", "rho_v", "rho_E"))
        for k in st:
            np.testing.assert_array_equal(st[k][g:-g, g:-g], ref[k][g:-g, g:-g][:, j0:j1],
                                          err_msg=f"{k} rows {j0}:{j1}")
    # the grid's totals are the sums over the slabs (other summation order: to rounding)
    np.testing.assert_allclose(sum(f.conservation_sums() for f in fluids),
                               one.conservation_sums(), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
def test_slabs_of_a_rectilinear_grid(cato_lib, precision):
    """Non-uniform rows: each slab gets its own y nodes; the rows beyond a cut take only their
    states from the neighbour (the metrics of interior cells are the slab's)."""
    cfg, prims = ic.riemann_quadrant(48, precision=precision, limiter="MLP3")
    xs = np.concatenate([np.linspace(0.0, 0.3, 21), np.linspace(0.3, 1.0, 29)[1:]])
    ys = np.concatenate([np.linspace(0.0, 0.6, 31), np.linspace(0.6, 1.0, 19)[1:]])
    one = Fluid(cfg).set_rectilinear(xs, ys).initialize(*prims)
    dts = [one.integrate()[0] for _ in range(STEPS)]
    parts = [slabs.slab_config(cfg, r, 3) for r in range(3)]
    fluids = [Fluid(c).set_rectilinear(xs, ys[j0:j1 + 1])
              .initialize(*slabs.slab_fields(cfg, prims, j0, j1)) for c, j0, j1 in parts]
    run = slabs.SlabRun(fluids, slabs.SlabComm(3, False))
    assert [run.step()[0] for _ in range(STEPS)] == dts
    g = cfg.ghost_layers()
    ref = one.state(("rho", "rho_E"))
    for f, (c, j0, j1) in zip(fluids, parts):
        st = f.state(("rho", "rho_E"))
        for k in st:
            np.testing.assert_array_equal(st[k][g:-g, g:-g], ref[k][g:-g, g:-g][:, j0:j1])


def test_slab_handles_refuse_the_whole_grid_entry_points(cato_lib):
    cfg, prims = ic.riemann_quadrant(32)
    c0, j0, j1 = slabs.slab_config(cfg, 0, 2)
    f = Fluid(c0).initialize(*slabs.slab_fields(cfg, prims, j0, j1))
    for call in (lambda: f.integrate(), lambda: f.run(0.1, 2), lambda: f.tune(1),
                 lambda: f.set_step_options(allow_subcycle=True)):
        with pytest.raises(CatoError) as e:
            call()
        assert e.value.code == 10
    with pytest.raises(CatoError):
        f.halo_export("-y")  # a physical side of slab 0
    with pytest.raises(CatoError):
        f.step_stage()  # no step open
    b = Batch(1, precision="fp64")
    with pytest.raises(Exception):
        b.add(dataclasses.replace(c0), slabs.slab_fields(cfg, prims, j0, j1))
    b.close()
