"""Input decks (mod_input.f90:194-445): parsing, defaults, validation, and the reference's own
integrated-test decks (read from the reference checkout when it is present)."""
import ctypes
import glob
import os

import numpy as np
import pytest

from fvleg_2d_gb300 import _lib
from fvleg_2d_gb300.deck import DeckError, parse_deck

DECK = """
[general]
title = 'uniform box'   ; a comment
[time]
max_time = .25d0
integration_strategy = "ssp_rk3"
cfl = 0.4
max_iterations = 100
[physics]
polytropic_index = 1.4
[scheme]
flux_solver = 'HLLC'
limiter = 'MLP5'
apply_low_mach_fix = .false.
[initial_conditions]
read_from_file = false
init_density = 1.2
init_x_velocity = 0.1
init_pressure = 2.5
[grid]
ni_nodes = 65
nj_nodes = 33
xmin = 0.0
xmax = 2.0
ymin = -0.5
ymax = 0.5
[boundary_conditions]
plus_x = 'outflow'
outflow_ambient_pressure = 2.0
minus_x = 'zero_gradient'
plus_y = 'symmetry'
minus_y = 'symmetry'
"""


def test_parse_values_and_defaults():
    d = parse_deck(DECK)
    assert d.title == "uniform box" and d.max_time == 0.25 and d.cfl == 0.4
    assert d.integration_strategy == "ssp_rk3" and d.max_iterations == 100
    assert d.flux_solver == "HLLC" and d.limiter == "MLP5" and d.n_ghost_layers == 3
    assert d.apply_low_mach_fix is False
    assert d.grid() == (64, 32, 2.0 / 64, 1.0 / 32)
    assert d.bc == {"+x": "outflow", "-x": "zero_gradient", "+y": "symmetry", "-y": "symmetry"}
    assert d.outflow_ambient_pressure == 2.0
    assert d.contour_interval_dt == 0.1  # deck default
    cfg = d.scheme()
    assert (cfg.ni, cfg.nj, cfg.gamma, cfg.ghost_layers()) == (64, 32, 1.4, 3)
    c = cfg.to_c()
    assert _lib.load(build_if_missing=True).cato_config_check(ctypes.byref(c)) == 0
    rho, u, v, p = d.initial_primitives(cfg)
    assert rho[3, 3] == 1.2 and u[3, 3] == 0.1 and v[3, 3] == 0.0 and p[3, 3] == 2.5
    assert rho[0, 0] == 0.0  # ghosts are left to the boundary conditions


@pytest.mark.parametrize("edit,msg", [
    (("limiter = 'MLP5'", "limiter = 'MLP5'\n[grid]\nn_ghost_layers = 2"), "ghost"),
    (("flux_solver = 'HLLC'", "flux_solver = 'FVLEG'"), "flux_solver"),
    (('integration_strategy = "ssp_rk3"', "integration_strategy = 'ssp_rk43'"), "no-op"),
    (("outflow_ambient_pressure = 2.0", ""), "outflow_ambient_pressure"),
])
def test_invalid_decks(edit, msg):
    text = DECK.replace(*edit)
    with pytest.raises(DeckError, match=msg):
        parse_deck(text).scheme()


# the reference checkout, when the environment variable REFERENCE names one
_REF = os.environ.get("REFERENCE", "")
REF_DECKS = sorted(glob.glob(os.path.join(_REF, "tests/integrated/*/input.ini"))) if _REF else []


@pytest.mark.skipif(not REF_DECKS, reason="reference checkout not present")
def test_reference_integrated_decks_parse():
    supported = 0
    for path in REF_DECKS:
        with open(path) as f:
            text = f.read()
        try:
            d = parse_deck(text)
        except DeckError as e:
            # a key read without a default is missing: cfgio stops the reference too
            # (cfgio_mod.f90 errexit) -- e.g. decks without [scheme] flux_solver
            assert "required" in str(e), (path, e)
            continue
        assert d.max_time > 0 and d.polytropic_index > 1, path
        try:
            cfg = d.scheme(ni=64, nj=32, dx=0.01, dy=0.01)
        except DeckError as e:  # M-AUSMPW+, pressure_input, ssp_rk43 decks
            assert any(k in str(e) for k in ("flux_solver", "boundary", "integration")), (path, e)
            continue
        c = cfg.to_c()
        assert _lib.load(build_if_missing=True).cato_config_check(ctypes.byref(c)) == 0, path
        supported += 1
    assert supported >= 15
    with open(os.path.join(os.path.dirname(REF_DECKS[0]), "..", "sod_1d", "input.ini")) as f:
        sod = parse_deck(f.read())
    assert (sod.flux_solver, sod.limiter, sod.integration_strategy) == ("Roe", "MLP5", "ssp_rk2")
    assert sod.bc["+x"] == "zero_gradient" and sod.bc["+y"] == "periodic" and sod.cfl == 0.1


PBC_DECK = """
[reference_state]
reference_length = 2.0
reference_density = 0.5
reference_velocity = 4.0
[time]
max_time = 0.05
integration_strategy = 'ssp_rk2'
[physics]
polytropic_index = 1.4
[scheme]
flux_solver = 'AUSMPW+'
[initial_conditions]
read_from_file = false
init_density = 1.0
init_pressure = 1.0
[grid]
ni_nodes = 11
nj_nodes = 6
xmin = 0
xmax = 1
ymin = 0
ymax = 0.5
[boundary_conditions]
plus_x = 'pressure_input'
minus_x = 'symmetry'
plus_y = 'symmetry'
minus_y = 'symmetry'
bc_density = 0.25
bc_pressure_input_file = 'drive.dat'
bc_pressure_scale_factor = 2.0
"""


def test_pressure_input_keys_and_table(tmp_path):
    from fvleg_2d_gb300.deck import nondim_factors, read_bc_pressure_table

    (tmp_path / "drive.dat").write_text("# time pressure density\n0.0 1.0d0 0.5\n"
                                        "1e-1 3.0 0.75\n0.2, 2.0, 1.0\nend of table\n")
    d = parse_deck(PBC_DECK)
    assert d.bc["+x"] == "pressure_input" and not d.apply_constant_bc_pressure
    t, p, rho = read_bc_pressure_table(d, str(tmp_path))
    f = nondim_factors(d)
    np.testing.assert_array_equal(t, np.array([0.0, 0.1, 0.2]) * (1.0 / (2.0 / 4.0)))
    np.testing.assert_array_equal(p, (np.array([1.0, 3.0, 2.0]) * (1.0 / (0.5 * 16.0))) * 2.0)
    np.testing.assert_array_equal(rho, (np.array([0.5, 0.75, 1.0]) * (1.0 / 0.5)) * 2.0)
    cfg = d.scheme()
    assert cfg.bc_density == 0.25 * f["density_to_dim"]
    const = parse_deck(PBC_DECK.replace("bc_pressure_input_file = 'drive.dat'",
                                        "apply_constant_bc_pressure = true\n"
                                        "constant_bc_pressure_value = 3.0"))
    assert const.scheme().constant_bc_pressure == 3.0 * f["press_to_nondim"]
    with pytest.raises(DeckError):
        parse_deck(PBC_DECK.replace("bc_pressure_input_file = 'drive.dat'", ""))


def test_fortran_es_editing():
    from fvleg_2d_gb300.deck import fortran_es

    assert fortran_es(1.23456e-3, 16, 6) == "    1.234560E-03"
    assert fortran_es(-0.5, 16, 6) == "   -5.000000E-01"
    assert fortran_es(0.0, 14, 4) == "    0.0000E+00"
    assert fortran_es(1e-120, 16, 6) == "    1.000000-120"  # three-digit exponent: no E
    assert fortran_es(2.5, 10, 3) == " 2.500E+00"


def test_run_history_files(tmp_path):
    """residual_hist.csv (mod_fluid.f90:244-246, 1207-1223), timing.csv and timing_summary.yaml
    (mod_timing.f90) in the reference's formats."""
    from fvleg_2d_gb300.deck import RunHistory

    h = RunHistory(str(tmp_path), t_to_dim=2.0)
    h.residual(1, 0.5, 0.25, [1e-3, 2e-4, 0.0, 3e-5])
    h.timing(1, 0.25)
    h.close()
    res = (tmp_path / "residual_hist.csv").read_text().splitlines()
    assert res[0] == "iteration,time,dt,rho,rho_u,rho_v,rho_E"
    assert res[1] == ("1,    1.000000E+00,    5.000000E-01,    1.000000E-03,    2.000000E-04,"
                      "    0.000000E+00,    3.000000E-05,")
    tim = (tmp_path / "timing.csv").read_text().splitlines()
    assert tim[0] == "iteration, elapsed_wall_time[sec], elapsed_cpu_time[sec], timestep[sec]"
    f = tim[1].split(", ")
    assert f[0] == "1" and len(f) == 4 and f[3].strip() == "2.5000E-01"
    summ = (tmp_path / "timing_summary.yaml").read_text().splitlines()
    assert len(summ) == 6 and summ[0].startswith("Total elapsed wall time [s]:")


def test_deck_reads_the_subcycle_keys():
    text = DECK.replace("[time]", "[time]\nallow_subcycle = .true.\nsubcycle_error_tolerance = 2e-4")
    d = parse_deck(text)
    assert d.allow_subcycle and d.subcycle_error_tolerance == 2e-4
