"""The FP64 oracle against the reference's own known-answer programs
(restated: the reference prints these values, it does not assert them) and
against dense state-vector simulation."""
import numpy as np
import pytest

from gates import (CX, CXREV, CZ, H, dense_apply1, dense_apply2, dense_entropy, dense_probs, dense_project,
                   xrot)
from oracle import mps_ref as R

LN2 = np.log(2.0)


def test_rotation_probs_and_postselection():
    """workspace/src/rotation_testing.rs:13-38: N=5, Const(2), XRot(3pi/5) on
    q2 then CX(2); p0 = cos^2(3pi/10), p1 = sin^2(3pi/10) on q2 and q3."""
    th = 3 * np.pi / 5
    m = R.MPS(5, R.Trunc.const(2))
    m.apply_unitary1(2, xrot(th))
    m.apply_unitary2(2, CX)
    p0, p1 = np.cos(th / 2) ** 2, np.sin(th / 2) ** 2
    for k in range(5):
        exp = [p0, p1] if k in (2, 3) else [1.0, 0.0]
        np.testing.assert_allclose(m.probs(k), exp, atol=1e-12)
    m0 = m.copy()
    assert abs(m0.measure_postsel_prob(2, 0) - p0) < 1e-12
    np.testing.assert_allclose(m0.probs(3), [1.0, 0.0], atol=1e-12)
    m1 = m.copy()
    assert abs(m1.measure_postsel_prob(2, 1) - p1) < 1e-12
    np.testing.assert_allclose(m1.probs(3), [0.0, 1.0], atol=1e-12)
    np.testing.assert_allclose(m1.probs(2), [0.0, 1.0], atol=1e-12)


@pytest.mark.parametrize("u,outcome,index", [(0.25, 0, 0), (0.75, 1, 12)])
def test_bell_doc_example(u, outcome, index):
    """mps.rs:43-95: n=4, H(0), CX(0), measure(0).  The doc comment there
    names e_0 or e_8, but CX on (0, 1) maps |10..> to |11..>, so outcome 1
    leaves e_12 (the example prints the vector, it asserts nothing)."""
    m = R.MPS(4, None)
    m.apply_unitary1(0, H)
    m.apply_unitary2(0, CX)
    p, prob = m.measure_prob(0, u)
    assert p == outcome and abs(prob - 0.5) < 1e-12
    psi = m.contract()
    exp = np.zeros(16, complex)
    exp[index] = 1.0
    assert np.allclose(np.abs(psi), np.abs(exp), atol=1e-12)


def test_density_matrix_two_qubits():
    """workspace/src/density_mat_testing.rs:87-221: two Haar unitaries with a
    post-selected measurement between them; joint probabilities against an
    explicit state calculation, probabilities summing to 1 within 1e-12."""
    rng = np.random.default_rng(5)
    z0 = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    z1 = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    u0, u1 = R.haar_from_ginibre(z0), R.haar_from_ginibre(z1)
    m = R.MPS(2, None)
    m.apply_unitary2(0, u0)
    p = m.probs(0)
    assert abs(p.sum() - 1.0) < 1e-12
    psi = np.zeros(4, complex)
    psi[0] = 1
    psi = u0 @ psi
    np.testing.assert_allclose(p, dense_probs(psi, 2, 0), atol=1e-12)
    for a in (0, 1):
        ma = m.copy()
        ma.measure_postsel_prob(0, a)
        ma.apply_unitary2(0, u1)
        pa = ma.probs(0)
        assert abs(pa.sum() - 1.0) < 1e-12
        psia = u1 @ dense_project(psi, 2, 0, a)
        np.testing.assert_allclose(pa, dense_probs(psia, 2, 0), atol=1e-12)


def _swap(m, k):
    m.apply_unitary2(k, CX)
    m.apply_unitary2(k, CXREV)
    m.apply_unitary2(k, CX)


def _ghz_state():
    """workspace/src/testing.rs:16-50 (N=5): H(0), CX between qubits 0 and 4
    through SWAP chains, then a Bell pair on (2, 3)."""
    n = 5
    m = R.MPS(n, None)
    m.apply_unitary1(0, H)
    for k in range(0, 3):
        _swap(m, k)
    m.apply_unitary2(3, CX)
    for k in (2, 1, 0):
        _swap(m, k)
    m.apply_unitary1(2, H)
    m.apply_unitary2(2, CX)
    return m


def test_ghz_swap_chain_entropies_and_outcomes():
    m = _ghz_state()
    ents = [m.entropy_vn(b) for b in range(4)]
    np.testing.assert_allclose(ents, [LN2, LN2, 2 * LN2, LN2], atol=1e-12)
    for u2, u3 in [(0.1, 0.9), (0.9, 0.1), (0.3, 0.3), (0.7, 0.7)]:
        mm = m.copy()
        a = mm.measure(2, u2)
        b = mm.measure(3, u3)
        assert a == b
        assert abs(mm.entropy_vn(2) - LN2) < 1e-12


def test_cluster_state_entropies():
    """workspace/src/state.rs:4-58: H on all, CZ(0), CZ(2), then alternating
    H / CZ(1) and H / CZ(0),CZ(2) rounds; entropy_vn(1) against dense."""
    n = 4
    m = R.MPS(n, None)
    psi = np.zeros(16, complex)
    psi[0] = 1
    assert abs(m.entropy_vn(1)) < 1e-14
    rounds = [[0, 2], [1], [0, 2], [1], [0, 2], [1], [0, 2], [1]]
    for czs in rounds:
        for k in range(n):
            m.apply_unitary1(k, H)
            psi = dense_apply1(psi, n, k, H)
        for k in czs:
            m.apply_unitary2(k, CZ)
            psi = dense_apply2(psi, n, k, CZ)
        e = m.entropy_vn(1)
        assert abs(e - dense_entropy(psi, n, 1)) < 1e-10
        assert min(abs(e - j * LN2) for j in range(3)) < 1e-10


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_dense_crosscheck_random_circuit(seed):
    """Haar brickwork + measurements without truncation: contract() equals the
    dense state vector; outcomes, probabilities and every bond's entropy equal
    the dense ones.  The last site is never measured here: see
    test_last_site_measurement_leaves_last_bond_stale."""
    n, depth, p = 8, 6, 0.3
    rng = np.random.default_rng(seed)
    m = R.MPS(n, None)
    psi = np.zeros(2 ** n, complex)
    psi[0] = 1
    for t in range(depth):
        gks = R.tile_q2(n, t % 2 == 1)
        gates = [R.haar_from_ginibre(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))) for _ in gks]
        meas = [k for k in range(n - 1) if rng.random() < p]
        us = rng.random(len(meas))
        rec = R.apply_bilayer(m, gks, gates, meas, us)
        for k, g in zip(gks, gates):
            psi = dense_apply2(psi, n, k, g)
        for (k, out, prob), u in zip(rec, us):
            pr = dense_probs(psi, n, k)
            assert out == (0 if u < pr[0] else 1)
            assert abs(prob - pr[out]) < 1e-10
            psi = dense_project(psi, n, k, out)
        phi = m.contract()
        assert abs(abs(np.vdot(phi, psi)) - 1.0) < 1e-10
        for b in range(n - 1):
            assert abs(m.entropy_vn(b) - dense_entropy(psi, n, b)) < 1e-9


def test_rank_rules():
    """process_svd rank selection (mps.rs:250-274) and the combined rule."""
    s = np.array([0.8, 0.5, 0.3, 1e-11, 1e-17, 0.0])
    s = s / np.linalg.norm(s)
    assert R.rank_rule(s, R.Trunc.none()) == 4  # > f64::EPSILON
    assert R.rank_rule(s, R.Trunc.const(2)) == 2
    assert R.rank_rule(s, R.Trunc.const(9)) == 4
    assert R.rank_rule(s, R.Trunc.const(0)) == 1
    assert R.rank_rule(s, R.Trunc.cut(1e-10)) == 3
    assert R.rank_rule(s, R.Trunc.cut(0.9)) == 1
    assert R.rank_rule(s, R.Trunc.both(2, 1e-10)) == 2
    assert R.rank_rule(s, R.Trunc.both(8, 1e-10)) == 3
    assert R.rank_rule(np.array([1.0, np.nan, 0.5]), R.Trunc.none()) == 1


def test_out_of_range_and_shape_errors():
    m = R.MPS(3, None)
    m.apply_unitary2(2, CX)  # k >= n-1: no-op
    m.apply_unitary1(5, H)  # no-op
    assert m.probs(3) is None and m.entropy_vn(2) is None and m.measure_prob(3, 0.5) is None
    with pytest.raises(ValueError):
        m.apply_unitary2(0, np.eye(2))
    one = R.MPS(1, None)
    np.testing.assert_allclose(one.probs(0), [1.0, 0.0])
    one.apply_unitary1(0, H)
    np.testing.assert_allclose(one.probs(0), [0.5, 0.5], atol=1e-15)
    with pytest.raises(ValueError):
        R.MPS(0, None)


def test_meas_layer_dedup_and_order():
    """apply_meas_prob_layer filters k < n, sorts and dedups; uniforms are
    consumed in ascending target order (mps.rs:2212-2245)."""
    a = _ghz_state()
    b = _ghz_state()
    ra = a.apply_meas_prob_layer([3, 2, 9, 3], [0.2, 0.6])
    rb = b.apply_meas_prob_layer([2, 3], [0.2, 0.6])
    assert [r[:2] for r in ra] == [r[:2] for r in rb]
    assert [r[0] for r in ra] == [2, 3]
    assert ra[0][1] == ra[1][1]
    assert a.apply_meas_prob_layer([], []) == []


def test_last_site_measurement_leaves_last_bond_stale():
    """Reference behaviour kept for parity: when the highest measured site is
    n-1, apply_meas_prob_layer refactors bonds last..n-2 (empty) and then
    n-3..0 (mps.rs:2246-2250), so bond n-2 keeps its pre-measurement Lambda.
    The contracted state is still the projected one."""
    n = 4
    m = R.MPS(n, None)
    m.apply_unitary1(2, H)
    m.apply_unitary2(2, CX)  # Bell pair on (2, 3)
    before = m.svals[n - 2].copy()
    psi = m.contract()
    rec = m.apply_meas_prob_layer([n - 1], [0.3])
    assert rec[0][:2] == (n - 1, 0)
    np.testing.assert_array_equal(m.svals[n - 2], before)  # stale: still (1/sqrt2, 1/sqrt2)
    proj = dense_project(psi, n, n - 1, 0)
    assert abs(abs(np.vdot(m.contract(), proj)) - 1.0) < 1e-12
    assert abs(m.entropy_vn(n - 2) - LN2) < 1e-12  # the true entropy is 0


def test_oracle_from_vector_factorize():
    """factorize (mps.rs:448-505): the contraction gives back the normalised
    vector; the bond-0 Schmidt values are those of the dense reshape; GHZ and
    product states have ranks 2 and 1."""
    rng = np.random.default_rng(2)
    n = 7
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    m = R.from_vector(psi)
    np.testing.assert_allclose(m.contract(), psi / np.linalg.norm(psi), atol=1e-13)
    for b in range(n - 1):
        s = np.linalg.svd((psi / np.linalg.norm(psi)).reshape(1 << (b + 1), -1), compute_uv=False)
        np.testing.assert_allclose(m.svals[b], s[: len(m.svals[b])], atol=1e-13)
    t = R.from_vector(psi, R.Trunc.const(3))
    assert [len(s) for s in t.svals] == [2, 3, 3, 3, 3, 2]
    ghz = np.zeros(1 << n)
    ghz[0] = ghz[-1] = 1
    assert [len(s) for s in R.from_vector(ghz).svals] == [2] * (n - 1)
    one = R.from_vector(np.array([0.6, 0.8j]))
    assert one.n == 1 and np.allclose(one.data[0].reshape(-1), [0.6, 0.8j])


def _two_time(state, mid_layers, x0, x1, post=None, us=None):
    """One run of workspace/src/sampling_testing.rs:66-132 on a copy of
    `state`: first layer, measurement of x0 (post-selected or sampled),
    remaining layers, then probs / a sampled measurement of x1."""
    s = state.copy()
    for k, u in mid_layers[0]:
        s.apply_unitary2(k, u)
    if post is not None:
        p0 = s.probs(x0)[post]
        s.measure_postsel_prob(x0, post)
        for layer in mid_layers[1:]:
            for k, u in layer:
                s.apply_unitary2(k, u)
        return p0 * s.probs(x1)
    a = s.measure(x0, us[0])
    for layer in mid_layers[1:]:
        for k, u in layer:
            s.apply_unitary2(k, u)
    return a, s.measure(x1, us[1])


def test_sampling_exact_two_time_probabilities_match_monte_carlo():
    """workspace/src/sampling_testing.rs: N=8, Const(6), 2N Haar layers, then
    the two-time joint distribution of Z at N/2 (after one more layer) and Z
    at N/2 (after two more): exact by post-selection, probabilities summing
    to 1 within 1e-12, against a seeded Monte-Carlo of sampled measurements
    (2000 runs, 5 sigma)."""
    n, dt = 8, 2
    x0 = x1 = n // 2
    rng = np.random.default_rng(10546)

    def layer(t):
        return [(k, R.haar_from_ginibre(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))))
                for k in R.tile_q2(n, t % 2 == 1)]

    init = [layer(t) for t in range(2 * n)]
    mid = [layer(t) for t in range(dt + 1)]
    state = R.MPS(n, R.Trunc.const(6))
    for lay in init:
        for k, u in lay:
            state.apply_unitary2(k, u)
    exact = np.array([_two_time(state, mid, x0, x1, post=a) for a in (0, 1)])  # [a][b]
    assert abs(exact.sum() - 1.0) < 1e-12
    counts = np.zeros((2, 2))
    runs = 2000
    urng = np.random.default_rng(7)
    for _ in range(runs):
        a, b = _two_time(state, mid, x0, x1, us=urng.random(2))
        counts[a, b] += 1
    freq = counts / runs
    sigma = np.sqrt(np.maximum(exact * (1 - exact), 1e-4) / runs)
    assert np.all(np.abs(freq - exact) < 5 * sigma), (freq, exact)
