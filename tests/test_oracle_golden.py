"""Pin the oracle to the reference's own known answers (tests/golden/reference_unit_vectors.json,
extracted from the reference's unit tests by tests/golden/make_golden.py) and to the Sod exact
solution; the GPU BC test at the end replays the same cases through the C-ABI."""
import json
import os

import numpy as np
import pytest

from fvleg_2d_gb300 import ic
from fvleg_2d_gb300.config import SchemeConfig

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "reference_unit_vectors.json")))


def simple_setup():
    """The simple.h5 fixture: 4x4 interior, 2 ghost layers, rho = u = v = p = data."""
    sg = GOLDEN["simple_grid"]
    ni, nj, ng = sg["ni"], sg["nj"], sg["n_ghost"]
    dx = (sg["xrange"][1] - sg["xrange"][0]) / ni
    dy = (sg["yrange"][1] - sg["yrange"][0]) / nj
    data = np.zeros((ni + 2 * ng, nj + 2 * ng), order="F")
    for j, row in sg["rows"].items():
        data[ng:ng + ni, int(j) - 1 + ng] = row
    return ni, nj, ng, dx, dy, data


def _index(expr: str, ni, nj, ng, axis: int):
    """Evaluate one reference index expression (left_ghost + 1, bottom:top, :) into a slice of
    the halo-padded numpy array."""
    names = {"left": 1, "right": ni, "bottom": 1, "top": nj, "left_ghost": 1 - ng,
             "right_ghost": ni + ng, "bottom_ghost": 1 - ng, "top_ghost": nj + ng}
    n = ni if axis == 0 else nj
    off = ng - 1
    if expr == ":":
        return slice(0, n + 2 * ng)
    if ":" in expr:
        a, b = expr.split(":")
        return slice(eval(a, {}, names) + off, eval(b, {}, names) + off + 1)
    return eval(expr, {}, names) + off


def _bc_cfg(ni, nj, ng, dx, dy, bc):
    return SchemeConfig(ni=ni, nj=nj, dx=dx, dy=dy, bc=bc, n_ghost=ng)


@pytest.mark.parametrize("case", GOLDEN["bc"]["cases"], ids=lambda c: c["test"])
def test_oracle_bc_matches_reference_unit_tests(oracle, case):
    ni, nj, ng, dx, dy, data = simple_setup()
    cfg = _bc_cfg(ni, nj, ng, dx, dy, {s: "zero_gradient" for s in ("+x", "+y", "-x", "-y")})
    f = {k: data.copy(order="F") for k in ("rho", "u", "v", "p")}
    do_corners = case["test"] == "test_periodic_all"  # all four input BCs periodic
    for bc_type, side in case["applied"]:
        oracle.apply_bc_side(cfg, side, bc_type, do_corners, f["rho"], f["u"], f["v"], f["p"])
    assert case["checks"], "no asserts extracted"
    for chk in case["checks"]:
        a, b = chk["index"]
        got = f[chk["field"]][_index(a, ni, nj, ng, 0), _index(b, ni, nj, ng, 1)]
        np.testing.assert_array_equal(np.atleast_1d(got), chk["expected"],
                                      err_msg=f"{case['test']} line {chk['line']}")


def test_oracle_limiters_match_reference(oracle):
    for name, pairs in GOLDEN["limiters"]["values"].items():
        for r, expected in pairs:
            assert oracle.limiter(name, r) == expected, (name, r)


def _tvd2_field(cfg, ng):
    col = GOLDEN["tvd2_none"]["column_values"]
    q = np.zeros(cfg.halo_shape, order="F")
    for i, val in col.items():
        q[int(i) + ng - 1, :] = val
    return q


def test_oracle_tvd2_edges_match_reference(oracle):
    """test_reconstruction.pf:145-148 (old cell-based API, limiter 'none'): at cell (2,2) the
    edge values are bottom 3.0, right 3.5, top 3.0, left 2.5; with minmod the slopes there are
    unlimited (r = 1), so the new edge-based arrays must hold the same values."""
    g = GOLDEN["tvd2_none"]
    cfg = SchemeConfig(ni=2, nj=4, dx=1.0, dy=1.0, limiter="minmod",
                       bc={s: "zero_gradient" for s in ("+x", "+y", "-x", "-y")})
    q = _tvd2_field(cfg, 2)
    ie, je = oracle.interpolate_edges(cfg, q)
    i, j = g["cell"]
    exp = dict(g["edge_values"])
    # i_edges(1:2, -1:ni, 0:nj): L of edge i+1/2 is cell i's right value; R of edge (i-1)+1/2 is
    # cell i's left value.  j_edges(1:2, 0:ni, -1:nj) likewise in j.
    assert ie[0, i + 1, j] == exp[2]
    assert ie[1, (i - 1) + 1, j] == exp[4]
    assert je[0, i, j + 1] == exp[3]
    assert je[1, i, (j - 1) + 1] == exp[1]


def test_oracle_quad_cell_matches_reference(oracle):
    g = GOLDEN["quad_cell"]
    m = oracle.quad_metrics(g["x"], g["y"])
    assert m["volume"] == g["volume"]
    assert list(m["edge_lengths"]) == g["edge_lengths"]
    np.testing.assert_array_equal(m["edge_norm_vectors"], np.array(g["edge_norm_vectors"]))


def test_grid_nodes_match_reference():
    g = GOLDEN["grid_nodes"]
    sg = GOLDEN["simple_grid"]
    x = ic.node_coordinates(sg["ni"], *sg["xrange"], sg["n_ghost"])
    y = ic.node_coordinates(sg["nj"], *sg["yrange"], sg["n_ghost"])
    np.testing.assert_array_equal(x, g["node_x"])
    for j, val in g["node_y"].items():
        assert y[int(j) + sg["n_ghost"] - 1] == val


def test_uniform_geometry_equals_quad_cell_of_nodes(oracle):
    """The uniform (dx, dy) geometry the kernels use equals the quad_cell_t metrics of the
    simple grid's node coordinates (integer-valued nodes: no rounding)."""
    sg = GOLDEN["simple_grid"]
    x = ic.node_coordinates(sg["ni"], *sg["xrange"], sg["n_ghost"])
    y = ic.node_coordinates(sg["nj"], *sg["yrange"], sg["n_ghost"])
    dx, dy = x[1] - x[0], y[1] - y[0]
    for i in range(len(x) - 1):
        for j in range(len(y) - 1):
            m = oracle.quad_metrics([x[i], x[i + 1], x[i + 1], x[i]], [y[j], y[j], y[j + 1], y[j + 1]])
            assert m["volume"] == dx * dy
            assert list(m["edge_lengths"]) == [dx, dy, dx, dy]
            assert (m["min_dx"], m["min_dy"]) == (dx, dy)


def _sod_exact(x, t, gamma=1.4, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), x0=0.5):
    """Exact Riemann solution (Toro, Riemann Solvers..., 2009, Ch. 4): density at x, time t."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = np.sqrt(gamma * pl / rl), np.sqrt(gamma * pr / rr)

    def fk(p, rk, pk, ck):
        if p > pk:
            ak, bk = 2.0 / ((gamma + 1) * rk), (gamma - 1) / (gamma + 1) * pk
            return (p - pk) * np.sqrt(ak / (p + bk))
        return 2 * ck / (gamma - 1) * ((p / pk) ** ((gamma - 1) / (2 * gamma)) - 1)

    lo, hi = 1e-8, 10.0
    for _ in range(200):  # bisection on the pressure function
        pm = 0.5 * (lo + hi)
        if fk(pm, rl, pl, cl) + fk(pm, rr, pr, cr) + (ur - ul) > 0:
            hi = pm
        else:
            lo = pm
    p_star = 0.5 * (lo + hi)
    u_star = 0.5 * (ul + ur) + 0.5 * (fk(p_star, rr, pr, cr) - fk(p_star, rl, pl, cl))
    g1 = (gamma - 1) / (gamma + 1)
    r_star_l = rl * (p_star / pl) ** (1 / gamma)  # left rarefaction
    r_star_r = rr * ((p_star / pr + g1) / (g1 * p_star / pr + 1))  # right shock
    s_shock = ur + cr * np.sqrt((gamma + 1) / (2 * gamma) * p_star / pr + (gamma - 1) / (2 * gamma))
    c_star_l = cl * (p_star / pl) ** ((gamma - 1) / (2 * gamma))
    s = (x - x0) / t
    rho = np.empty_like(s)
    head, tail = ul - cl, u_star - c_star_l
    for k, sk in enumerate(s):
        if sk < head:
            rho[k] = rl
        elif sk < tail:
            rho[k] = rl * (2 / (gamma + 1) + g1 / cl * (ul - sk)) ** (2 / (gamma - 1))
        elif sk < u_star:
            rho[k] = r_star_l
        elif sk < s_shock:
            rho[k] = r_star_r
        else:
            rho[k] = rr
    return rho


@pytest.mark.parametrize("flux", ["AUSMPW+", "M-AUSMPW+"])
def test_oracle_sod_against_exact_solution(oracle, flux):
    """Physical sanity bound (tests/integrated/sod_1d compares against an exact Riemann solver):
    the 400x40 Sod run at t ~ 0.2 is within 1 % L1 of the exact density and y-uniform."""
    cfg, prims = ic.sod(flux_solver=flux)
    f = oracle.OracleFluid(cfg)
    f.set_primitive(*prims)
    f.run(0.2)
    rho = f.state()["rho"][2:-2, 2:-2]
    assert np.abs(rho - rho[:, :1]).max() == 0.0
    xc = ic.cell_centres(cfg.ni, 0.0, 1.0, 2)[2:-2]
    exact = _sod_exact(xc, f.time)
    l1 = np.abs(rho[:, 0] - exact).mean() / np.abs(exact).mean()
    assert l1 < 0.01, l1


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in GOLDEN["bc"]["cases"] if len(c["applied"]) == 4],
                         ids=lambda c: c["test"])
def test_gpu_bc_matches_reference_unit_tests(cato_lib, case):
    """Through cato_gpu_solve, which writes the BC-filled ghosts back like the reference's
    intent(inout) primitives: cases whose reference test applies all four sides."""
    from fvleg_2d_gb300.fluid import FluxSolver

    ni, nj, ng, dx, dy, data = simple_setup()
    bc = {side: t for t, side in case["applied"]}
    cfg = _bc_cfg(ni, nj, ng, dx, dy, bc)
    f = {k: data.copy(order="F") for k in ("rho", "u", "v", "p")}
    FluxSolver(cfg).solve(f["rho"], f["u"], f["v"], f["p"])
    for chk in case["checks"]:
        a, b = chk["index"]
        got = f[chk["field"]][_index(a, ni, nj, ng, 0), _index(b, ni, nj, ng, 1)]
        np.testing.assert_array_equal(np.atleast_1d(got), chk["expected"],
                                      err_msg=f"{case['test']} line {chk['line']}")
