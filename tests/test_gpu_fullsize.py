"""The bench workload at full size (N=64, chi_max=256, cutoff 1e-10, p cycling
0.05..0.30, mixed precision), where the FP64 oracle is too slow to follow:
152 trajectories (one per SM) for 15 brickwork layers, until the middle
bonds saturate at chi_max, checked through size-independent properties.

* the measurement rule (mps.rs:1427-1447): outcome 0 exactly when the
  uniform is below p0, the reported probability is that outcome's, every
  listed site is measured once, in ascending order;
* the Schmidt form after every layer of work: Lambda on every bond sorted
  descending, positive, sum of squares 1, at most chi_max values, as many as
  the bond dimension;
* the reported half-chain entropy equals -sum s^2 ln s^2 of that bond's
  Lambda (mps.rs:1251-1261);
* each trajectory's results are bit-identical when it runs in a batch of
  two instead of 152 (the executor's fixed per-trajectory reduction order,
  whatever the schedule does with the other trajectories).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P_LIST = (0.05, 0.10, 0.15, 0.20, 0.30)
SEED = 20261203


def _layers(pkg, ids, t, n):
    return [pkg.gen_layer(SEED, i, t, n, P_LIST[i % len(P_LIST)]) for i in ids]


def test_full_size_invariants(pkg):
    n, chi, cut, B, depth = 64, 256, 1e-10, 152, 15
    b = pkg.Batch([n] * B, [pkg.Trunc.both(chi, cut)] * B, "mixed")
    ids = list(range(B))
    all_recs, all_ents = [], []
    for t in range(depth):
        layers = _layers(pkg, ids, t, n)
        recs, ents = b.step(ids, layers)
        all_recs.append(recs)
        all_ents.append(np.array(ents))
        for i in ids:
            _, _, mk, us = layers[i]
            assert [k for (k, _, _) in recs[i]] == [int(k) for k in mk]
            for (k, o, pr), u in zip(recs[i], us):
                assert 0.0 < pr <= 1.0 + 1e-9, (t, i, k, pr)
                p0 = pr if o == 0 else 1.0 - pr
                if abs(p0 - u) > 1e-6:
                    assert (o == 0) == (u < p0), (t, i, k, o, u, p0)
    assert b.device_status() == 0
    widest = 0
    for i in ids:
        dims = b.bond_dims(i)
        widest = max(widest, int(dims.max()))
        for bd in range(n - 1):
            s = b.svals(i, bd)
            assert len(s) == dims[bd] and 1 <= len(s) <= chi, (i, bd, len(s), dims[bd])
            assert np.all(s > 0) and np.all(np.diff(s) <= 1e-15), (i, bd)
            assert abs(float(np.sum(s * s)) - 1.0) < 1e-9, (i, bd)
        s = b.svals(i, n // 2 - 1)
        s2 = s * s
        assert abs(all_ents[-1][i] - float(-(s2 * np.log(s2)).sum())) < 1e-9, i
    assert widest == chi, widest  # the bench's saturated regime was reached

    # the same two trajectories alone in a batch of two: bit-identical
    pick = [0, 77]
    b2 = pkg.Batch([n] * 2, [pkg.Trunc.both(chi, cut)] * 2, "mixed")
    for t in range(depth):
        recs, ents = b2.step([0, 1], _layers(pkg, pick, t, n))
        for j, i in enumerate(pick):
            assert recs[j] == all_recs[t][i], (t, i)
            assert ents[j] == all_ents[t][i], (t, i)
    for j, i in enumerate(pick):
        for bd in range(n - 1):
            np.testing.assert_array_equal(b2.svals(j, bd), b.svals(i, bd))
    assert b2.device_status() == 0
