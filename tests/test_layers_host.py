"""Host logic of the workspace layer drivers (tensor-net_gb300/layers.py) on
the CPU, against a recording fake of the state: gates first, then one
single-site measurement per entry in list order (each with its own sweep in
the real state), one uniform per random measurement, and the probe filter
that keeps only the target's measurements (workspace/lib/haar.rs:103-206)."""
import numpy as np
import pytest


class FakeState:
    def __init__(self):
        self.calls = []

    def apply_unitary2(self, k, m):
        self.calls.append(("u2", k))

    def measure_prob(self, k, u):
        self.calls.append(("m", k, u))
        return (1 if u > 0.5 else 0, 0.25)

    def measure(self, k, u):
        return self.measure_prob(k, u)[0]

    def measure_postsel_prob(self, k, p):
        self.calls.append(("ps", k, p))
        return 0.75

    def measure_postsel(self, k, p):
        self.measure_postsel_prob(k, p)

    def probs(self, k):
        self.calls.append(("probs", k))
        return np.array([0.4, 0.6])


def test_main_layer_order_and_uniforms(pkg):
    from tensor_net_gb300 import layers
    from tensor_net_gb300.gates import Meas
    st = FakeState()
    outs, probs = layers.apply_main_layer_probs(
        st, [(0, np.eye(4)), (2, np.eye(4))], [Meas.rand(3), Meas.proj(1, 1), Meas.rand(0)], [0.9, 0.1])
    assert st.calls == [("u2", 0), ("u2", 2), ("m", 3, 0.9), ("ps", 1, 1), ("m", 0, 0.1)]
    assert [(o.k, o.outcome) for o in outs] == [(3, 1), (1, 1), (0, 0)]
    assert probs == [(3, 0.25), (1, 0.75), (0, 0.25)]
    assert [(o.k, o.outcome) for o in layers.apply_main_layer(FakeState(), [], [Meas.rand(2)], [0.2])] == [(2, 0)]
    with pytest.raises(ValueError):
        layers.apply_main_layer(FakeState(), [], [Meas.rand(2), Meas.rand(3)], [0.2])


def test_probe_layer_keeps_only_the_target(pkg):
    from tensor_net_gb300 import layers
    from tensor_net_gb300.gates import Meas
    st = FakeState()
    outs, pr = layers.apply_probe_layer(st, [(1, np.eye(4))], [Meas.rand(2), Meas.proj(5, 0), Meas.rand(5)],
                                        target=5, us=[0.7])
    assert st.calls == [("u2", 1), ("ps", 5, 0), ("m", 5, 0.7), ("probs", 5)]
    assert [(o.k, o.outcome) for o in outs] == [(5, 0), (5, 1)] and pr == (0.4, 0.6)
    st = FakeState()
    outs, pr = layers.apply_probe_layer(st, [], [Meas.rand(2), Meas.rand(4)], None, us=[0.1, 0.8])
    assert [(o.k, o.outcome) for o in outs] == [(2, 0), (4, 1)] and pr is None


def _bare_mps(pkg, n, record):
    """An MPS object without a device handle whose leaf methods record calls."""
    m = object.__new__(pkg.MPS)
    m._h = None
    m.n = n

    def aml(ks, us=None, posts=None):
        record.append(("layer", list(ks), None if posts is None else list(posts)))
        return [(k, p if p is not None else 0, 0.5) for k, p in zip(ks, posts or [None] * len(ks))]

    m.apply_meas_prob_layer = aml
    m.apply_unitary2 = lambda k, op: record.append(("u2", k, np.asarray(op)))
    return m


def test_postsel_layer_filter_and_multi_product(pkg):
    rec = []
    m = _bare_mps(pkg, 8, rec)
    # invalid quantum numbers and sites are dropped before the de-duplication (mps.rs:1623-1635)
    m.measure_postsel_prob_layer([(6, 2), (6, 1), (1, 0), (12, 0)])
    assert rec[-1] == ("layer", [6, 1], [1, 0])
    assert m.measure_postsel_prob_layer([(9, 0), (3, 5)]) == []
    # apply_unitary2_multi multiplies ops[-1] ... ops[0] (mps.rs:1404-1413)
    rng = np.random.default_rng(0)
    ops = [rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)) for _ in range(3)]
    m.apply_unitary2_multi(2, ops)
    np.testing.assert_allclose(rec[-1][2], ops[2] @ ops[1] @ ops[0])
    n_before = len(rec)
    m.apply_unitary2_multi(7, [np.eye(3)])  # out of range: nothing, not even the shape check
    assert len(rec) == n_before
    with pytest.raises(pkg.TnError):
        m.apply_unitary2_multi(1, [np.eye(4), np.eye(2)])
    assert len(rec) == n_before
