"""workspace/src/sampling_testing.rs on the GPU path: the two-time joint
distribution of Z at N/2 after one and after two more Haar layers, from an
N=8, Const(6) state after 2N layers.  Exact (post-selection) probabilities
match the oracle's to 1e-10 and sum to 1 within 1e-12; sampled runs fed the
same uniforms as the oracle give the same outcomes (ties |p - u| < 1e-9
aside); 2000 sampled runs match the exact distribution within 5 sigma."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _layers(pkg, ref, n, dt):
    rng = np.random.default_rng(10546)

    def layer(t):
        return [(k, ref.haar_from_ginibre(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))))
                for k in ref.tile_q2(n, t % 2 == 1)]

    return [layer(t) for t in range(2 * n)], [layer(t) for t in range(dt + 1)]


def _run(state, mid, x0, x1, clone, post=None, us=None):
    s = clone(state)
    for k, u in mid[0]:
        s.apply_unitary2(k, u)
    if post is not None:
        p0 = s.probs(x0)[post]
        s.measure_postsel_prob(x0, post)
        for layer in mid[1:]:
            for k, u in layer:
                s.apply_unitary2(k, u)
        return p0 * np.asarray(s.probs(x1))
    a = s.measure(x0, us[0])
    for layer in mid[1:]:
        for k, u in layer:
            s.apply_unitary2(k, u)
    return a, s.measure(x1, us[1])


def test_two_time_distribution(pkg, ref):
    n, dt = 8, 2
    x0 = x1 = n // 2
    init, mid = _layers(pkg, ref, n, dt)
    g = pkg.MPS.new_qubits(n, pkg.Trunc.const(6), "f64")
    r = ref.MPS(n, ref.Trunc.const(6))
    for lay in init:
        for k, u in lay:
            g.apply_unitary2(k, u)
            r.apply_unitary2(k, u)
    ex_g = np.array([_run(g, mid, x0, x1, lambda s: s.clone(), post=a) for a in (0, 1)])
    ex_r = np.array([_run(r, mid, x0, x1, lambda s: s.copy(), post=a) for a in (0, 1)])
    assert abs(ex_g.sum() - 1.0) < 1e-12
    np.testing.assert_allclose(ex_g, ex_r, atol=1e-10)
    urng = np.random.default_rng(7)
    counts = np.zeros((2, 2))
    runs = 2000
    for i in range(runs):
        us = urng.random(2)
        a, b = _run(g, mid, x0, x1, lambda s: s.clone(), us=us)
        counts[a, b] += 1
        if i < 200:  # the same uniforms through the oracle: the same outcomes
            assert (a, b) == _run(r, mid, x0, x1, lambda s: s.copy(), us=us), i
    freq = counts / runs
    sigma = np.sqrt(np.maximum(ex_g * (1 - ex_g), 1e-4) / runs)
    assert np.all(np.abs(freq - ex_g) < 5 * sigma), (freq, ex_g)
    assert g.device_status() == 0
