"""The oracle's energy source term (source_t, mod_source.f90:260-425) against a direct Python
transcription: the deposition column from the critical density, the input value from the table
or the constant, each geometry; plus the energy budget of a uniform source and the deck keys."""
import math

import numpy as np
import pytest

from conftest import random_prims
from fvleg_2d_gb300.config import EnergySource, SchemeConfig

PER = {"+x": "periodic", "-x": "periodic", "+y": "periodic", "-y": "periodic"}
TABLE = (np.array([0.0, 0.3, 1.0]), np.array([2.0, 5.0, 1.0]), np.array([0.9, 1.1, 1.3]))


def _cfg(ni=24, nj=10, **kw):
    return SchemeConfig(ni=ni, nj=nj, dx=1.0 / ni, dy=0.5 / nj, bc=PER, gamma=1.4, cfl=0.4,
                        flux_solver="HLLC", limiter="van_leer", **kw)


def _interp(t, f, x):
    n = len(t)
    il = n - 2 if x >= t[-1] else (0 if x < t[0] else max(k for k in range(n - 1) if t[k] <= x))
    q1 = (x - t[il]) / (t[il + 1] - t[il])
    return (1.0 - q1) * f[il] + q1 * f[il + 1]


def _powi(x, n):
    y = x if n % 2 else 1.0
    n >>= 1
    while n:
        x = x * x
        if n % 2:
            y = y * x
        n >>= 1
    return y


def _field(cfg, src, rho, time, xn, yn):
    """get_source_field after find_deposition_location, transcribed."""
    cx = [(xn[i + 1] + xn[i]) / 2.0 for i in range(cfg.ni)]
    cy = [(yn[j + 1] + yn[j]) / 2.0 for j in range(cfg.nj)]
    crit = _interp(*src.table[::2], time) if src.table else 0.0
    x0 = 0.0
    for i in range(cfg.ni - 1, -1, -1):
        if np.any(rho[i, :] > crit):
            x0 = cx[i]
            break
    if src.table is None:
        p_in = src.constant_value
    else:
        p_in = _interp(src.table[0], src.table[1], time) if time <= max(src.table[0]) else 0.0
    p_in = p_in * src.multiplier
    q = np.zeros((cfg.ni, cfg.nj))
    if abs(p_in) > 0.0:
        for i in range(cfg.ni):
            for j in range(cfg.nj):
                x, y = cx[i], cy[j]
                if src.geometry == "uniform":
                    q[i, j] = p_in
                elif src.geometry == "constant_xy":
                    if x < src.xhi and x > src.xlo and y < src.yhi and x > src.ylo:
                        q[i, j] = p_in
                elif src.geometry == "1d_gaussian":
                    if abs(x - x0) < src.fwhm_x * 5:
                        a = ((x - x0) * (x - x0)) / (2 * (src.fwhm_x * src.fwhm_x))
                        q[i, j] = p_in * math.exp(-_powi(a, src.gaussian_order))
                elif x < x0:
                    q[i, j] = p_in * math.exp(-math.pow(x / x0, 1.5)) / math.exp(-1.0)
                else:
                    q[i, j] = p_in * math.exp(-1e4 * (((x - x0) / x0) * ((x - x0) / x0)))
    return q


SOURCES = [
    EnergySource("uniform", constant_value=0.7, multiplier=2.0),
    EnergySource("constant_xy", multiplier=1.5, xlo=0.2, xhi=0.6, ylo=0.1, yhi=0.4, table=TABLE),
    EnergySource("1d_gaussian", fwhm_x=0.05, gaussian_order=2, table=TABLE),
    EnergySource("1d_gaussian", constant_value=3.0, fwhm_x=0.08, gaussian_order=1),
    EnergySource("decay", table=TABLE),
]


@pytest.mark.parametrize("k", range(len(SOURCES)))
@pytest.mark.parametrize("time", [0.0, 0.2, 0.7, 1.5])
def test_field_matches_transcription(oracle, k, time):
    cfg = _cfg()
    src = SOURCES[k]
    prims = random_prims(cfg, np.random.default_rng(k))
    g = cfg.ghost_layers()
    f = oracle.OracleFluid(cfg)
    xn = np.cumsum(np.concatenate([[0.0], 0.5 + np.random.default_rng(9).random(cfg.ni)]))
    xn = xn / xn[-1]
    yn = np.linspace(0.0, 0.5, cfg.nj + 1)
    f.set_rectilinear(xn, yn)
    f.set_primitive(*prims)
    f.set_time(time, 0)
    f.set_energy_source(src)
    got = f.source_field()
    want = _field(cfg, src, prims[0][g:-g, g:-g], time, xn, yn)
    np.testing.assert_array_equal(got, want)


def test_uniform_source_energy_budget(oracle):
    """A periodic box heated uniformly: the energy total grows by q x area x dt per step (the
    flux divergence telescopes), mass stays."""
    cfg = _cfg()
    f = oracle.OracleFluid(cfg)
    f.set_primitive(*random_prims(cfg, np.random.default_rng(3)))
    f.set_energy_source(EnergySource("uniform", constant_value=0.25))
    area = 1.0 * 0.5
    for _ in range(5):
        e0, m0 = f.conservation_sums()[3], f.conservation_sums()[0]
        assert f.integrate() == 0
        e1, m1 = f.conservation_sums()[3], f.conservation_sums()[0]
        assert abs((e1 - e0) - 0.25 * area * f.last_dt) <= 1e-12 * abs(e0)
        assert abs(m1 - m0) <= 1e-13 * abs(m0)


def test_deck_source_keys(tmp_path):
    from fvleg_2d_gb300.deck import DeckError, energy_source, nondim_factors, parse_deck

    deck_text = """
[reference_state]
reference_length = 2.0
reference_density = 0.5
reference_velocity = 4.0
[time]
max_time = 1
integration_strategy = 'ssp_rk3'
[physics]
polytropic_index = 1.4
[scheme]
flux_solver = 'AUSMPW+'
[initial_conditions]
initial_condition_file = 'x.npz'
[source_terms]
enable_source_terms = true
source_term_type = 'energy'
geometry = '1d_gaussian'
source_file = 'laser.dat'
source_scale_factor = 3.0
gaussian_fwhm_x = 0.1
gaussian_order = 2
"""
    (tmp_path / "laser.dat").write_text("# t q rho_c\n0 1e10 0.1\n1e-9 2e10 0.2\n")
    d = parse_deck(deck_text)
    src = energy_source(d, str(tmp_path))
    f = nondim_factors(d)
    assert src.geometry == "1d_gaussian" and src.gaussian_order == 2 and src.multiplier == 3.0
    assert src.fwhm_x == 0.1 * f["len_to_nondim"]
    np.testing.assert_array_equal(src.table[1], np.array([1e10, 2e10]) * f["pow_to_nondim"])
    np.testing.assert_array_equal(src.table[2], np.array([0.1, 0.2]) * f["density_to_nondim"])
    with pytest.raises(DeckError):
        energy_source(parse_deck(deck_text.replace("'energy'", "'force'")), str(tmp_path))
    with pytest.raises(ValueError):
        EnergySource("2d_gaussian").to_c()
