"""The config-4 request stream (no GPU): Poisson arrivals, side distribution, flux mix."""
import math

import numpy as np

from fvleg_2d_gb300.serve import SERVING_FLUXES, make_requests


def test_request_stream_statistics():
    reqs = make_requests(2000, rate=100.0, seed=1)
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert abs(gaps.mean() - 0.01) < 0.001  # mean inter-arrival 1/rate
    sides = np.array([r.n for r in reqs])
    assert sides.min() >= 128 and sides.max() <= 2048 and np.all(sides % 16 == 0)
    # log-uniform: the median side is near the geometric mean of the range
    assert abs(math.log(np.median(sides)) - 0.5 * (math.log(128) + math.log(2048))) < 0.15
    counts = {f: sum(r.flux == f for r in reqs) for f in SERVING_FLUXES}
    assert min(counts.values()) > 300
    assert all(0.05 <= r.t_end <= 0.3 for r in reqs)
    assert len({r.seed for r in reqs}) == 2000
