"""Fixed gate sets through the GPU path (apply_gate / apply_circuit /
apply_uni / apply_bilayer_ops, mps.rs:2044-2126, circuit.rs:624-659) against
the FP64 oracle and dense state vectors: float64, 1e-10."""
import numpy as np
import pytest

from gates import dense_apply1, dense_apply2

pytestmark = pytest.mark.gpu

LN2 = np.log(2.0)


def _random_circuit(g, n, count, rng):
    G = g.Gate
    out = []
    for _ in range(count):
        kind = rng.integers(0, 12)
        k1, k2 = int(rng.integers(0, n)), int(rng.integers(0, n - 1))
        a, b, c = rng.uniform(-np.pi, np.pi, 3)
        out.append([G.U(k1, a, b, c), G.H(k1), G.X(k1), G.Z(k1), G.S(k1), G.SInv(k1), G.XRot(k1, a),
                    G.ZRot(k1, b), G.CX(k2), G.CXRev(k2), G.CZ(k2), G.Haar2(k2)][kind])
    return out


def test_random_fixed_gate_circuit_matches_oracle_and_dense(pkg, ref):
    from tensor_net_gb300 import gates as g
    n = 6
    circ = _random_circuit(g, n, 60, np.random.default_rng(11))
    m = pkg.MPS.new_qubits(n, None, "f64")
    r = ref.MPS(n, None)
    psi = np.zeros(1 << n, complex)
    psi[0] = 1
    rng = np.random.default_rng(5)
    for gate in circ:
        k, mat = gate.into_matrix(rng)
        m.apply_uni(g.Uni.mat(k, mat))
        if gate.is_q1():
            r.apply_unitary1(k, mat)
            psi = dense_apply1(psi, n, k, mat)
        else:
            r.apply_unitary2(k, mat)
            psi = dense_apply2(psi, n, k, mat)
    a = m.contract()
    assert abs(abs(np.vdot(a, psi)) - 1.0) < 1e-10
    for b in range(n - 1):
        np.testing.assert_allclose(m.svals(b), r.svals[b][: len(m.svals(b))], atol=1e-10)
        assert abs(m.entropy_vn(b) - r.entropy_vn(b)) < 1e-10
    assert m.device_status() == 0


def test_ghz_and_cluster_from_fixed_gates(pkg):
    from tensor_net_gb300 import gates as g
    n = 8
    ghz = pkg.MPS.new_qubits(n, None, "f64")
    ghz.apply_circuit([g.Gate.H(0)] + [g.Gate.CX(k) for k in range(n - 1)])
    for b in range(n - 1):
        assert abs(ghz.entropy_vn(b) - LN2) < 1e-12
    for k in range(n):
        np.testing.assert_allclose(ghz.probs(k), [0.5, 0.5], atol=1e-12)
    cl = pkg.MPS.new_qubits(n, None, "f64")
    cl.apply_circuit([g.Gate.H(k) for k in range(n)] + [g.Gate.CZ(k) for k in range(n - 1)])
    for b in range(n - 1):
        assert abs(cl.entropy_vn(b) - LN2) < 1e-12
    # the reference's X gate is the identity (gate.rs:649-658): |0...0> stays put
    x = pkg.MPS.new_qubits(4, None, "f64")
    x.apply_circuit([g.Gate.X(k) for k in range(4)])
    for k in range(4):
        np.testing.assert_allclose(x.probs(k), [1.0, 0.0], atol=1e-15)


def test_uni_shapes_and_out_of_range(pkg):
    from tensor_net_gb300 import gates as g
    m = pkg.MPS.new_qubits(4, None, "f64")
    with pytest.raises(pkg.TnError) as e:
        m.apply_uni(g.Uni.mat(0, np.eye(3)))
    assert e.value.status == -5
    # out-of-range qubits are a no-op (mps.rs:2040-2043)
    m.apply_gate(g.Gate.H(9)).apply_gate(g.Gate.CZ(3))
    np.testing.assert_allclose(m.probs(0), [1.0, 0.0], atol=1e-15)


def test_bilayer_ops_with_rand_and_proj_matches_oracle(pkg, ref):
    from tensor_net_gb300 import gates as g
    n = 8
    m = pkg.MPS.new_qubits(n, pkg.Trunc.both(16, 1e-12), "f64")
    r = ref.MPS(n, ref.Trunc.both(16, 1e-12))
    for t in range(10):
        gk, gs, mk, us = pkg.gen_layer(21, 0, t, n, 0.0)
        unis = [g.Uni.mat(int(k), u) for k, u in zip(gk, gs)]
        meas = [g.Meas.rand(1), g.Meas.proj(4, 0), g.Meas.rand(6)] if t % 3 == 2 else []
        u = np.array([0.37, 0.0, 0.81])[: len(meas)]
        outs, probs = m.apply_bilayer_ops(unis, meas, u)
        for k, gm in zip(gk, gs):
            r.apply_unitary2(int(k), gm)
        want = r.apply_meas_prob_layer([x.k for x in meas], u, posts=[x.outcome for x in meas])
        assert [(o.k, o.outcome) for o in outs] == [(k, o) for (k, o, _) in want]
        for (k, p), (_, _, p2) in zip(probs, want):
            assert abs(p - p2) < 1e-10
    for b in range(n - 1):
        assert abs(m.entropy_vn(b) - r.entropy_vn(b)) < 1e-10
    assert m.device_status() == 0


def test_layer_variants_multi_and_reset_match_the_oracle(pkg, ref):
    """measure_layer / measure_prob_layer / measure_postsel_(prob_)layer
    (mps.rs:1519-1657), apply_unitary2_multi (1393-1414), max_bond_dim_idx
    (1235-1239) and measure_reset (2278-2286) against the oracle."""
    from tensor_net_gb300 import gates as g
    n = 8
    m = pkg.MPS.new_qubits(n, None, "f64")
    r = ref.MPS(n, None)
    layers = pkg.gen_trajectory(31, 0, n, 4, 0.0)
    for (gk, gs, _, _) in layers:
        for k, u in zip(gk, gs):
            m.apply_unitary2(int(k), u)
            r.apply_unitary2(int(k), u)
    # measure_layer over unsorted duplicates and an out-of-range target
    ks, us = [5, 2, 9, 5], [0.3, 0.8]
    out = m.measure_prob_layer(ks, us)
    want = r.apply_meas_prob_layer(ks, us)
    assert [o for o, _ in out] == [o for (_, o, _) in want]
    for (_, p), (_, _, p2) in zip(out, want):
        assert abs(p - p2) < 1e-10
    # post-selected layer: (k, p) pairs, invalid p and k dropped before the de-duplication
    probs = m.measure_postsel_prob_layer([(6, 2), (6, 1), (1, 0), (12, 0)])
    want = r.apply_meas_prob_layer([1, 6], None, posts=[0, 1])  # the oracle's posts follow the sorted targets
    assert len(probs) == 2 and all(abs(a - b[2]) < 1e-10 for a, b in zip(probs, want))
    # apply_unitary2_multi = one apply_unitary2 of the product
    ops = [pkg.haar_u4(pkg.ginibre(3, 0, 0, j)) for j in range(3)]
    m.apply_unitary2_multi(3, ops)
    r.apply_unitary2(3, ops[2] @ ops[1] @ ops[0])
    for b in range(n - 1):
        assert abs(m.entropy_vn(b) - r.entropy_vn(b)) < 1e-10
    with pytest.raises(pkg.TnError):
        m.apply_unitary2_multi(3, [np.eye(4), np.eye(2)])
    m.apply_unitary2_multi(7, [np.eye(3)])  # out of range: no-op before the shape check
    dims = [m.bond_dim(b) for b in range(n - 1)]
    assert m.max_bond_dim_idx() == max(i for i, d in enumerate(dims) if d == max(dims))
    # measure_reset: the reference's XMAT is the identity, so outcome 1 stays 1
    o = m.measure_reset(4, 0.999999)
    if o == 1:
        np.testing.assert_allclose(m.probs(4), [0.0, 1.0], atol=1e-12)
    assert m.apply_op(g.Meas.proj(4, o)) == o
    assert m.apply_op(g.Uni.of_gate(g.Gate.H(0))) is None
    assert m.device_status() == 0


def test_workspace_layer_drivers_match_the_oracle(pkg, ref):
    """apply_main_layer(_probs) / apply_probe_layer (workspace/lib/haar.rs:
    103-206): gates, then one measurement at a time with a full sweep each,
    in list order; the oracle composed from the same single-site calls."""
    from tensor_net_gb300 import layers
    from tensor_net_gb300.gates import Meas
    n = 8
    m = pkg.MPS.new_qubits(n, pkg.Trunc.both(16, 1e-12), "f64")
    r = ref.MPS(n, ref.Trunc.both(16, 1e-12))
    for t in range(6):
        gk, gs, _, _ = pkg.gen_layer(41, 0, t, n, 0.0)
        unis = list(zip(gk, gs))
        meas = [Meas.rand(5), Meas.proj(2, t % 2), Meas.rand(0)] if t % 2 else [Meas.rand(3)]
        us = [0.41, 0.77][: sum(x.is_rand() for x in meas)]
        outs, probs = layers.apply_main_layer_probs(m, unis, meas, us)
        for k, u in unis:
            r.apply_unitary2(int(k), u)
        it = iter(us)
        want = []
        for x in meas:
            if x.is_rand():
                o, p = r.measure_prob(x.k, next(it))
            else:
                o, p = x.outcome, r.measure_postsel_prob(x.k, x.outcome)
            want.append((x.k, o, p))
        assert [(y.k, y.outcome) for y in outs] == [(k, o) for (k, o, _) in want]
        for (k, p), (_, _, p2) in zip(probs, want):
            assert abs(p - p2) < 1e-10
    gk, gs, _, _ = pkg.gen_layer(41, 0, 6, n, 0.0)
    outs, pr = layers.apply_probe_layer(m, list(zip(gk, gs)), [Meas.rand(1), Meas.rand(4)], target=4, us=[0.5])
    for k, u in zip(gk, gs):
        r.apply_unitary2(int(k), u)
    o = r.measure(4, 0.5)
    assert [(y.k, y.outcome) for y in outs] == [(4, o)]  # only the target's measurement, as the reference's filter
    np.testing.assert_allclose(pr, r.probs(4), atol=1e-10)
    for b in range(n - 1):
        assert abs(m.entropy_vn(b) - r.entropy_vn(b)) < 1e-10
