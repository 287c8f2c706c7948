"""GPU path (through the C ABI, batched) against the committed FP64 golden
trajectories: float64 to 1e-9 (entropies, probabilities, Schmidt values),
mixed to 1e-4; outcomes identical except at |p - u| < 1e-9 ties."""
import numpy as np
import pytest

from golden_cases import load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [("f64", 1e-9), ("mixed", 1e-4)])
def test_batch_matches_golden(pkg, prec, tol):
    cases = load()
    b = pkg.Batch([c["n"] for c in cases], [pkg.Trunc.both(c["chi"], c["cutoff"]) for c in cases], prec)
    depth = max(c["depth"] for c in cases)
    for t in range(depth):
        live = [i for i, c in enumerate(cases) if t < c["depth"]]
        recs, ents = b.step(live, [cases[i]["layers"][t] for i in live])
        for j, i in enumerate(live):
            c = cases[i]
            gold = c["recs"][t]
            for (k, o, p), (k2, o2, p2) in zip(recs[j], gold):
                assert k == k2
                u = c["layers"][t][3][[x[0] for x in gold].index(k)]
                assert o == o2 or abs(p2 - u) < 1e-9 or abs((1 - p2) - u) < 1e-9, (c["name"], t, k)
                assert abs(p - p2) < tol, (c["name"], t, k, p, p2)
            assert abs(ents[j] - c["entropy"][t]) < tol, (c["name"], t)
    for i, c in enumerate(cases):
        for bd in range(c["n"] - 1):
            g, r = b.svals(i, bd), c["svals"][bd]
            k = min(len(g), len(r))
            keep = r[:k] > (1e-6 if prec == "f64" else 1e-3)
            assert np.count_nonzero(r > (1e-6 if prec == "f64" else 1e-3)) == np.count_nonzero(keep)
            np.testing.assert_allclose(g[:k][keep], r[:k][keep], rtol=tol * 10)
    assert b.device_status() == 0
