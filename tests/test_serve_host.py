"""The serving workload's request stream on the CPU (serve.poisson_requests):
Poisson arrivals at the stated mean rate over the window, N log-uniform in
[16, 128], chi_max from {64, 128, 256, 512}, p uniform in [0.02, 0.3], depth
uniform in [2N, 4N], seeded and reproducible."""
import math

import numpy as np


def test_poisson_request_stream_has_the_specified_mix(pkg):
    reqs = pkg.poisson_requests(200.0, 60.0, 7)
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) > 0) and t[-1] <= 60.0
    assert abs(len(reqs) - 12000) < 5 * math.sqrt(12000)  # Poisson count at 200/s over 60 s
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 200.0) < 0.05 / 200.0
    ns = np.array([r["n"] for r in reqs])
    assert ns.min() >= 16 and ns.max() <= 128
    # log-uniform: the median sits near the geometric mean sqrt(16 * 128) ~ 45
    assert abs(np.median(ns) - math.sqrt(16 * 128)) < 3
    assert set(r["chi"] for r in reqs) == {64, 128, 256, 512}
    ps = np.array([r["p"] for r in reqs])
    assert ps.min() >= 0.02 and ps.max() <= 0.3
    assert all(2 * r["n"] <= r["depth"] <= 4 * r["n"] for r in reqs)
    assert [r["traj"] for r in reqs] == list(range(len(reqs)))
    assert pkg.poisson_requests(200.0, 60.0, 7) == reqs
