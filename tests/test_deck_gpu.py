"""A whole deck through the GPU path (run_deck: the main.f90 loop of cato.x input.ini) against the
oracle running the same configuration: identical step count, time and state."""
import numpy as np
import pytest

from conftest import interior
from fvleg_2d_gb300.deck import load_initial_condition, parse_deck, run_deck, t_to_nondim
from test_icfile_cpu import layered_nodes, make_file, uniform_nodes

pytestmark = pytest.mark.gpu

DECK = """
[general]
title = 'outflow box'
[time]
max_time = 0.02
integration_strategy = 'ssp_rk3'
cfl = 0.4
[physics]
polytropic_index = 1.4
[scheme]
flux_solver = 'M-AUSMPW+'
limiter = 'MLP3'
[initial_conditions]
read_from_file = false
init_density = 1.2
init_x_velocity = 0.3
init_pressure = 2.5
[grid]
ni_nodes = 49
nj_nodes = 25
xmin = 0.0
xmax = 1.0
ymin = 0.0
ymax = 0.5
[boundary_conditions]
plus_x = 'outflow'
outflow_ambient_pressure = 2.0
minus_x = 'zero_gradient'
plus_y = 'symmetry'
minus_y = 'symmetry'
"""


def test_run_deck_matches_oracle(oracle, cato_lib):
    deck = parse_deck(DECK)
    fluid, steps = run_deck(deck)
    cfg = deck.scheme()
    ref = oracle.OracleFluid(cfg)
    ref.set_primitive(*deck.initial_primitives(cfg))
    n = ref.run(deck.max_time)
    assert steps == n and fluid.time == ref.time
    a, b = ref.state(), fluid.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(interior(cfg, b[k]), interior(cfg, a[k]), err_msg=k)
    # the outflow boundary at 2.0 < 2.5 drives an expansion into the box
    assert interior(cfg, b["rho"]).min() < 1.2


FILE_DECK = """
[reference_state]
reference_length = 0.5
reference_density = 1.5
reference_velocity = 2.0e5
[time]
max_time = 1.5e-6
integration_strategy = 'ssp_rk2'
cfl = 0.5
[physics]
polytropic_index = 1.6667
[scheme]
flux_solver = 'SLAU2'
limiter = 'MLP5'
[initial_conditions]
read_from_file = true
initial_condition_file = 'layered.npz'
[boundary_conditions]
plus_x = 'zero_gradient'
minus_x = 'symmetry'
plus_y = 'periodic'
minus_y = 'periodic'
"""


def test_run_deck_from_layered_file_matches_oracle(oracle, cato_lib, tmp_path):
    """A file-driven deck (read_from_file) on a pycato layered grid: the GPU run and the oracle
    on the file's rectilinear grid agree bit for bit."""
    ng = 3
    xn = layered_nodes([(0.05, 12), (0.2, 20), (0.75, 40)], ng)
    make_file(str(tmp_path / "layered.npz"), xn, uniform_nodes(24, 0.0, 0.3, ng), ng, seed=4)
    deck = parse_deck(FILE_DECK)
    fluid, steps = run_deck(deck, base_dir=str(tmp_path))
    ic = load_initial_condition(deck, str(tmp_path))
    assert ic.uniform is None
    cfg = deck.scheme(*ic.scheme_grid())
    ref = oracle.OracleFluid(cfg)
    ref.set_rectilinear(ic.x_nodes, ic.y_nodes)
    ref.set_primitive(*ic.primitives)
    n = ref.run(deck.max_time * t_to_nondim(deck))
    assert steps == n > 3 and fluid.time == ref.time
    a, b = ref.state(), fluid.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(interior(cfg, b[k]), interior(cfg, a[k]), err_msg=k)


def test_run_deck_pressure_input_table_matches_oracle(oracle, cato_lib, tmp_path):
    """A deck with a tabulated +x pressure input (bc_pressure_input_file): the GPU run and the
    oracle with the same scaled table agree bit for bit (correctly rounded inlet powers)."""
    from test_deck_cpu import PBC_DECK
    from fvleg_2d_gb300.deck import read_bc_pressure_table

    (tmp_path / "drive.dat").write_text("# t p rho\n0.0 4.0 0.5\n0.02 12.0 0.75\n"
                                        "0.05 6.0 1.0\n")
    deck = parse_deck(PBC_DECK)
    fluid, steps = run_deck(deck, base_dir=str(tmp_path))
    cfg = deck.scheme()
    ref = oracle.OracleFluid(cfg)
    ref.set_bc_table(*read_bc_pressure_table(deck, str(tmp_path)))
    ref.set_primitive(*deck.initial_primitives(cfg))
    with oracle.pow_mode("cr"):  # the inlet's powers as the device rounds them
        n = ref.run(deck.max_time * t_to_nondim(deck))
    assert steps == n > 3 and fluid.time == ref.time
    a, b = ref.state(), fluid.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(interior(cfg, b[k]), interior(cfg, a[k]), err_msg=k)


def test_run_deck_with_contours_matches_oracle(oracle, cato_lib, tmp_path):
    """main.f90's loop with contour output every contour_interval_dt (its own clock snaps to
    the output times): the same iterations and the same state as the oracle driven through the
    same loop, and one contour per output time with the state of that iteration."""
    from fvleg_2d_gb300.deck import main_loop, nondim_factors

    text = DECK.replace("[general]", "[io]\ncontour_interval_dt = 0.005\n[general]")
    deck = parse_deck(text)
    assert deck.contour_interval_dt == 0.005
    out = tmp_path / "results"
    fluid, steps = run_deck(deck, results_dir=str(out))
    cfg = deck.scheme()

    class Ref:
        def __init__(self):
            self.f = oracle.OracleFluid(cfg)
            self.f.set_primitive(*deck.initial_primitives(cfg))
            self.last_dt = 0.0

        @property
        def time(self):
            return self.f.time

        def step(self, dt):
            ec = self.f.integrate(dt)
            self.last_dt = self.f.last_dt
            return ec

        def state(self, names):
            return self.f.state()

    ref = Ref()
    n = main_loop(deck, ref, ref.step)
    assert steps == n and fluid.time == ref.time
    a, b = ref.f.state(), fluid.state()
    for k in ("rho", "rho_u", "rho_v", "rho_E"):
        np.testing.assert_array_equal(interior(cfg, b[k]), interior(cfg, a[k]), err_msg=k)
    from fvleg_2d_gb300 import h5lite

    files = sorted(p.name for p in out.iterdir() if p.suffix == ".h5")
    assert files[0] == "step_0000000.h5" and len(files) >= 4
    with h5lite.H5File(str(out / files[-1])) as last:
        assert last.read("density").shape == (cfg.nj, cfg.ni)
        t_dim = float(last.read("time"))
    f = nondim_factors(deck)
    assert 0 < t_dim <= fluid.time * (1.0 / f["t_to_nondim"])
