"""tn_mps_apply_unitary2_noalloc: applying a two-qubit gate without any device
allocation.

Callers that must not allocate GPU memory at the moment they apply a gate --
a runtime that fixes its whole device memory plan at start-up, or one that
applies gates while other work is being captured into a CUDA graph -- use
this entry point instead of tn_mps_apply_unitary2.  Its scratch is a fixed
4.5 MiB array compiled into the library, so it must give the same state as the
ordinary entry point, call after call, at every bond capacity it accepts, it
must allocate nothing, and it must refuse handles whose bond capacity needs
more scratch than that array holds.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-9, "mixed": 1e-4, "df": 1e-9}  # the parity tolerances of the other GPU tests


def _noalloc(pkg, m, k, op):
    a = np.ascontiguousarray(np.asarray(op, dtype=np.complex128))
    buf = a.view(np.float64).reshape(-1).copy()
    return pkg.lib().tn_mps_apply_unitary2_noalloc(m._h, int(k), buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                   a.shape[0], a.shape[1])


def _same_state(ref, new, n, tol):
    for b in range(n - 1):
        sr, sn = ref.svals(b), new.svals(b)
        assert len(sr) == len(sn), (b, len(sr), len(sn))
        assert np.max(np.abs(sr - sn)) < tol, b
    for q in range(n):
        assert np.max(np.abs(ref.probs(q) - new.probs(q))) < tol, q


@pytest.mark.parametrize("prec,n,chi,cap", [("f64", 10, 16, 0), ("mixed", 10, 16, 0), ("df", 10, 16, 0),
                                            ("mixed", 18, 256, 256), ("f64", 18, 191, 191)])
def test_noalloc_matches_apply_unitary2(pkg, prec, n, chi, cap):
    """Two calls in a row give the state of the ordinary entry point, also at
    the largest bond capacity each precision accepts (mixed: 256 of the
    workloads; float64: 191)."""
    trunc = pkg.Trunc.both(chi, 1e-12)
    ref = pkg.MPS.new_qubits(n, trunc, prec, cap)
    new = pkg.MPS.new_qubits(n, trunc, prec, cap)
    # the same entangled starting state through the ordinary entry point
    for (gk, gates, _, _) in pkg.gen_trajectory(3, 0, n, 5, 0.0):
        for k, g in zip(gk, gates):
            ref.apply_unitary2(k, g)
            new.apply_unitary2(k, g)
    gates = pkg.gen_layer(4, 0, 0, n, 0.0)[1]
    # two calls in a row (neighbouring bonds, so the second reads what the first wrote)
    for k, g in [(n // 2 - 1, gates[0]), (n // 2, gates[1])]:
        ref.apply_unitary2(k, g)
        assert _noalloc(pkg, new, k, g) == 0
        _same_state(ref, new, n, TOL[prec])
    assert new.device_status() == 0


def test_noalloc_allocates_nothing(pkg):
    """Device free memory is unchanged across noalloc calls on a fresh handle
    (after one call that sets the entry point up on this device)."""
    import torch
    n = 12
    m = pkg.MPS.new_qubits(n, pkg.Trunc.both(32, 1e-12), "mixed")
    gates = pkg.gen_layer(5, 0, 0, n, 0.0)[1]
    assert _noalloc(pkg, m, 0, gates[0]) == 0
    assert m.device_status() == 0  # (reads the status word: waits for the handle's stream)
    free0 = torch.cuda.mem_get_info()[0]
    for i, g in enumerate(gates):
        assert _noalloc(pkg, m, (2 * i + 1) % (n - 1), g) == 0
    assert m.device_status() == 0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_refuses_bad_input_and_keeps_the_state(pkg):
    n = 8
    m = pkg.MPS.new_qubits(n, pkg.Trunc.both(16, 1e-12), "f64")
    for (gk, gates, _, _) in pkg.gen_trajectory(9, 0, n, 3, 0.0):
        for k, g in zip(gk, gates):
            m.apply_unitary2(k, g)
    before = [m.probs(q).copy() for q in range(n)]
    bad = np.eye(4, dtype=np.complex128)
    bad[1, 2] = np.nan
    assert _noalloc(pkg, m, 3, bad) == -6  # TN_ERR_INVALID_ARG, as tn_mps_apply_unitary2
    for q in range(n):
        np.testing.assert_array_equal(m.probs(q), before[q])
    assert m.device_status() == 0


def test_noalloc_rejects_what_the_fixed_scratch_cannot_hold(pkg):
    big = pkg.MPS.new_qubits(20, pkg.Trunc.both(192, 1e-10), "f64")  # chi cap 192 in float64: above 4.5 MiB
    assert _noalloc(pkg, big, 3, np.eye(4)) == -9  # TN_ERR_CAPACITY
    assert "4.5 MiB" in pkg.lib().tn_last_error().decode()
    big2 = pkg.MPS.new_qubits(20, pkg.Trunc.both(271, 1e-10), "mixed")
    assert _noalloc(pkg, big2, 3, np.eye(4)) == -9
    small = pkg.MPS.new_qubits(6, None, "f64")
    assert _noalloc(pkg, small, 1, np.eye(2)) == -5  # TN_ERR_OPERATOR_SHAPE, as tn_mps_apply_unitary2
    assert _noalloc(pkg, small, 5, np.eye(4)) == 0  # out of range: silent no-op, as the reference
