"""Serving loop: requests admitted while others run give exactly the result they give alone,
FP64 requests give the oracle's state, step count and error code (the random-circle initial
states make some schemes fail with a negative pressure or density, in the reference too), and
admission respects the HBM budget."""
import numpy as np
import pytest

from conftest import interior
from fvleg_2d_gb300.serve import Server, make_requests, run_alone

pytestmark = pytest.mark.gpu


def test_each_result_same_alone_and_in_mix(cato_lib):
    reqs = make_requests(10, rate=400.0, seed=3, side=(32, 96), t_end=(0.01, 0.03))
    srv = Server(precision="mixed", budget_gb=120.0, capacity=16, chunk_steps=8,
                 keep_results=True)
    stats = srv.serve(reqs)
    srv.close()
    assert len(stats.completed) == len(reqs) and stats.censored == 0
    overlapped = sum(1 for r in reqs for o in reqs
                     if r is not o and o.admitted < r.finished and r.admitted < o.finished)
    assert overlapped > 0, "requests should share the GPU"
    for r in reqs:
        ref = run_alone(r)
        assert r.steps == ref["steps"] and r.error_code == ref["error_code"]
        for k in ("rho", "rho_u", "rho_v", "rho_E"):
            np.testing.assert_array_equal(r.result[k], ref[k], err_msg=f"request {r.rid} {k}")


def test_fp64_requests_match_oracle(cato_lib, oracle):
    reqs = make_requests(10, rate=400.0, seed=3, side=(32, 96), t_end=(0.01, 0.03),
                         precision="fp64")
    srv = Server(precision="fp64", budget_gb=120.0, capacity=16, chunk_steps=8,
                 keep_results=True)
    stats = srv.serve(reqs)
    srv.close()
    assert len(stats.completed) == len(reqs)
    n_failed = 0
    for r in reqs:
        cfg, prims = r.config_and_ic()
        f = oracle.OracleFluid(cfg)
        f.set_primitive(*prims)
        ec = 0
        while f.time < r.t_end and not ec:
            ec = f.integrate()
        assert (r.steps, r.error_code) == (f.iteration, ec), f"request {r.rid} {r.flux}"
        n_failed += ec != 0
        if ec == 0:
            ref = f.state()
            for k in ("rho", "rho_u", "rho_v", "rho_E"):
                np.testing.assert_array_equal(interior(cfg, r.result[k]), interior(cfg, ref[k]),
                                              err_msg=f"request {r.rid} {k}")
    assert 0 < n_failed < len(reqs)  # both outcomes are covered


def test_admission_respects_budget(cato_lib):
    reqs = make_requests(6, rate=1000.0, seed=4, side=(48, 64), t_end=(0.01, 0.02))
    from fvleg_2d_gb300.batch import instance_bytes

    need = {r.rid: instance_bytes(r.config_and_ic()[0]) for r in reqs}
    budget = 2.5 * max(need.values())
    srv = Server(precision="mixed", budget_gb=budget / 1e9, capacity=16, chunk_steps=4)
    stats = srv.serve(reqs)
    srv.close()
    assert len(stats.completed) == 6
    # at every admission the resident instances fit the budget, and the budget did bind
    peak = 0
    for r in reqs:
        live = [o for o in reqs if o.admitted <= r.admitted < o.finished]
        assert sum(need[o.rid] for o in live) <= budget
        peak = max(peak, len(live))
    assert peak < len(reqs)
