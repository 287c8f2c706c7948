"""tn_mps_apply_unitary2_noalloc: applying a two-qubit gate without any device
allocation.

Callers that must not allocate GPU memory at the moment they apply a gate --
a runtime that fixes its whole device memory plan at start-up, or one that
applies gates while other work is being captured into a CUDA graph -- use
this entry point instead of tn_mps_apply_unitary2.  Its scratch is a fixed
4 MiB array compiled into the library, so it must give the same state as the
ordinary entry point, call after call, and it must refuse handles whose bond
capacity needs more scratch than that array holds.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-9, "mixed": 1e-4}  # the parity tolerances of the other GPU tests


def _noalloc(pkg, m, k, op):
    a = np.ascontiguousarray(np.asarray(op, dtype=np.complex128))
    buf = a.view(np.float64).reshape(-1).copy()
    return pkg.lib().tn_mps_apply_unitary2_noalloc(m._h, int(k), buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                   a.shape[0], a.shape[1])


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_noalloc_matches_apply_unitary2(pkg, prec):
    n, chi = 10, 16
    trunc = pkg.Trunc.both(chi, 1e-12)
    ref = pkg.MPS.new_qubits(n, trunc, prec)
    new = pkg.MPS.new_qubits(n, trunc, prec)
    # the same entangled starting state through the ordinary entry point
    for (gk, gates, _, _) in pkg.gen_trajectory(3, 0, n, 5, 0.0):
        for k, g in zip(gk, gates):
            ref.apply_unitary2(k, g)
            new.apply_unitary2(k, g)
    gates = pkg.gen_layer(4, 0, 0, n, 0.0)[1]
    # two calls in a row (neighbouring bonds, so the second reads what the first wrote)
    for k, g in [(4, gates[0]), (5, gates[1])]:
        ref.apply_unitary2(k, g)
        assert _noalloc(pkg, new, k, g) == 0
        for b in range(n - 1):
            sr, sn = ref.svals(b), new.svals(b)
            assert len(sr) == len(sn), (b, len(sr), len(sn))
            assert np.max(np.abs(sr - sn)) < TOL[prec], b
        for q in range(n):
            assert np.max(np.abs(ref.probs(q) - new.probs(q))) < TOL[prec], q
    assert new.device_status() == 0


def test_noalloc_rejects_what_the_fixed_scratch_cannot_hold(pkg):
    big = pkg.MPS.new_qubits(20, pkg.Trunc.both(256, 1e-10), "f64")  # chi cap 256 in float64: more than 4 MiB
    assert _noalloc(pkg, big, 3, np.eye(4)) == -9  # TN_ERR_CAPACITY
    assert "4 MiB" in pkg.lib().tn_last_error().decode()
    small = pkg.MPS.new_qubits(6, None, "f64")
    assert _noalloc(pkg, small, 1, np.eye(2)) == -5  # TN_ERR_OPERATOR_SHAPE, as tn_mps_apply_unitary2
    assert _noalloc(pkg, small, 5, np.eye(4)) == 0  # out of range: silent no-op, as the reference
