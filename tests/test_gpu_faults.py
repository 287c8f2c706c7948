"""Failure handling that needs a device but never faults it: refused
allocations come back as TN_ERR_OOM and leave the library usable; poisoned
inputs (non-finite gate entries or uniforms) are refused before any device
work; the device error word stays clear."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_allocation_failure_is_an_error_and_recoverable(pkg):
    # a bond capacity of 2^20 at n = 64 asks for petabytes: cudaMalloc refuses
    with pytest.raises(pkg.TnError) as e:
        pkg.MPS.new_qubits(64, None, "f64", chi_cap=1 << 20)
    assert e.value.status == -8
    with pytest.raises(pkg.TnError) as e:
        pkg.Batch([64] * 4, [pkg.Trunc.const(1 << 20)] * 4, "f64", chi_caps=[1 << 20] * 4)
    assert e.value.status == -8
    m = pkg.MPS.new_qubits(6, None, "f64")  # the library still works
    m.apply_unitary2(0, np.eye(4))
    assert abs(m.entropy_vn(0)) < 1e-14 and m.device_status() == 0


def test_non_finite_inputs_are_refused(pkg):
    m = pkg.MPS.new_qubits(6, None, "f64")
    bad = np.eye(4, dtype=complex)
    bad[1, 2] = np.nan
    for call in (lambda: m.apply_unitary2(1, bad), lambda: m.apply_unitary1(0, np.array([[1, 0], [0, np.inf]])),
                 lambda: m.measure_prob(2, np.nan),
                 lambda: m.apply_bilayer([0], [bad], [], []),
                 lambda: m.apply_bilayer([0], [np.eye(4)], [3], [np.nan]),
                 lambda: m.apply_meas_prob_layer([1, 2], [0.5, np.inf])):
        with pytest.raises(pkg.TnError) as e:
            call()
        assert e.value.status == -6
    np.testing.assert_allclose(m.probs(1), [1.0, 0.0], atol=1e-15)  # state untouched
    b = pkg.Batch([6, 6], [pkg.Trunc.const(8)] * 2, "mixed")
    gk, g, mk, us = pkg.gen_layer(1, 0, 0, 6, 0.5)
    g2 = g.copy()
    g2[0, 0, 0] = np.nan
    with pytest.raises(pkg.TnError) as e:
        b.step([0], [(gk, g2, mk, us)])
    assert e.value.status == -6
    if len(mk):
        with pytest.raises(pkg.TnError) as e:
            b.step([0], [(gk, g, mk, np.full(len(mk), np.nan))])
        assert e.value.status == -6
    recs, ents = b.step([0, 1], [(gk, g, mk, us)] * 2)  # a good step still runs
    assert recs[0] == recs[1] and b.device_status() == 0


def test_queue_wait_limit_runs_out_and_is_reported(pkg):
    """A CTA's wait for a pushed sweep item is bounded: with one sweep slot
    that no work item ever fills and a 5 ms limit, the launch still ends,
    the batch reports ST_QUEUE_WAIT (bit 16), the real trajectories' results
    are those of an ordinary batch, and the next ordinary step is clean."""
    ns = [10, 12, 9]
    truncs = [pkg.Trunc.both(16, 1e-12)] * 3
    test, ref = pkg.Batch(ns, truncs, "mixed"), pkg.Batch(ns, truncs, "mixed")
    layers = [pkg.gen_layer(41, i, 0, n, 0.2) for i, n in enumerate(ns)]
    for b in (test, ref):
        b.step([0, 1, 2], layers)  # sizes the step buffers for three trajectories
    assert test.device_status() == 0
    test.set_queue_wait(5_000_000, 1)  # 5 ms, one phantom sweep slot
    layers = [pkg.gen_layer(41, i, 1, n, 0.2) for i, n in enumerate(ns)]
    r_t, e_t = test.step([0, 1], layers[:2])
    r_r, e_r = ref.step([0, 1], layers[:2])
    assert test.device_status() & 16
    assert r_t == r_r and list(e_t) == list(e_r)
    test.set_queue_wait(0, 0)
    layers = [pkg.gen_layer(41, i, 2, n, 0.2) for i, n in enumerate(ns)]
    r_t, e_t = test.step([0, 1, 2], layers)
    r_r, e_r = ref.step([0, 1, 2], layers)
    assert test.device_status() == 0 and ref.device_status() == 0
    assert r_t == r_r and list(e_t) == list(e_r)
