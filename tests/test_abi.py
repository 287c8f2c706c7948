"""The C ABI library without a GPU: it loads, exports every entry point that
include/tn_mps.h declares, fails loudly when no device is present, and its
host-only parts (seeded inputs, Haar construction) are right."""
import ctypes
import pathlib
import re

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def header_functions():
    txt = (ROOT / "include" / "tn_mps.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tn_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.lib()
    names = header_functions()
    assert len(names) >= 40
    for name in names:
        assert hasattr(lib, name), name
    from tensor_net_gb300 import _lib
    assert set(_lib.SIGNATURES) == set(names)


def test_library_is_in_tree_and_sm103a(pkg):
    so = pkg.library_path()
    assert so.exists() and so.parent.parent.name == "tensor-net_gb300"
    build = (ROOT / "tensor-net_gb300" / "build.py").read_text()
    assert "arch=compute_103a,code=sm_103a" in build


def test_status_strings(pkg):
    lib = pkg.lib()
    assert lib.tn_status_string(-5).decode() == "error in operator application: incorrect shape"
    assert lib.tn_status_string(-1).decode().startswith("error in MPS creation")


def test_no_device_fails_loudly(pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.TnError) as e:
        pkg.MPS.new_qubits(4)
    assert "NO_DEVICE" in str(e.value)
    with pytest.raises(pkg.TnError):
        pkg.Batch([4, 4])


def test_empty_system_is_an_error(pkg):
    lib = pkg.lib()
    h = ctypes.c_void_p()
    assert lib.tn_mps_new_qubits(0, None, 0, 0, ctypes.byref(h)) == -1


def test_import_argument_errors(pkg):
    """tn_mps_import's shape checks come before any device work."""
    lib = pkg.lib()
    h = ctypes.c_void_p()
    U = ctypes.POINTER(ctypes.c_uint32)
    D = ctypes.POINTER(ctypes.c_double)
    g = np.zeros(64)
    lam = np.ones(4)
    for chi, want in (([1, 2, 1], None), ([2, 2, 1], -4), ([1, 0, 1], -4), ([1, 2, 2], -4)):
        c = np.array(chi, np.uint32)
        r = lib.tn_mps_import(2, c.ctypes.data_as(U), g.ctypes.data_as(D), lam.ctypes.data_as(D), None, 0, 0,
                              ctypes.byref(h))
        if want is not None:
            assert r == want, (chi, r)
    assert lib.tn_mps_import(0, None, None, None, None, 0, 0, ctypes.byref(h)) == -1
    c = np.array([1, 2, 1], np.uint32)
    bad = g.copy()
    bad[3] = np.nan
    assert lib.tn_mps_import(2, c.ctypes.data_as(U), bad.ctypes.data_as(D), lam.ctypes.data_as(D), None, 0, 0,
                             ctypes.byref(h)) == -6
    assert lib.tn_mps_import(2, c.ctypes.data_as(U), g.ctypes.data_as(D), lam.ctypes.data_as(D), None, 0, 1,
                             ctypes.byref(h)) == -9  # a bond of 2 above chi_cap 1


def test_from_vector_argument_errors(pkg):
    """from_vector's MPSError cases (mps.rs:517-530) come before any device work."""
    lib = pkg.lib()
    h = ctypes.c_void_p()
    psi = np.zeros(2 * 8)
    p = psi.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert lib.tn_mps_from_vector(0, p, 0, None, 0, 0, ctypes.byref(h)) == -1   # EmptySystem
    assert lib.tn_mps_from_vector(3, p, 6, None, 0, 0, ctypes.byref(h)) == -4   # StateIncompatibleShape
    assert lib.tn_mps_from_vector(21, p, 1 << 21, None, 0, 0, ctypes.byref(h)) == -6
    assert lib.tn_mps_from_vector(3, None, 8, None, 0, 0, ctypes.byref(h)) == -6
    with pytest.raises(pkg.TnError) as e:
        pkg.MPS.from_vector(np.ones(6))
    assert e.value.status == -4


def test_haar_matches_independent_qr(pkg, ref):
    """tn_haar_u4 (MGS QR) equals gate::haar's Householder QR + phase fix."""
    for site in range(6):
        z = pkg.ginibre(11, 3, 5, site)
        u = pkg.haar_u4(z)
        np.testing.assert_allclose(u, ref.haar_from_ginibre(z), atol=1e-13)
        np.testing.assert_allclose(u.conj().T @ u, np.eye(4), atol=1e-13)


def test_generated_layer_structure(pkg, ref):
    n, p = 17, 0.25
    tot_meas = 0
    for t in range(40):
        gk, g, mk, us = pkg.gen_layer(123, 4, t, n, p)
        assert list(gk) == ref.tile_q2(n, t % 2 == 1)
        assert g.shape == (len(gk), 4, 4)
        assert np.all(np.diff(mk.astype(int)) > 0) and np.all(mk < n)
        assert np.all((us >= 0) & (us < 1))
        tot_meas += len(mk)
        gk2, g2, mk2, us2 = pkg.gen_layer(123, 4, t, n, p)  # deterministic
        assert np.array_equal(g, g2) and np.array_equal(us, us2)
    rate = tot_meas / (40 * n)
    assert 0.15 < rate < 0.35
    # other trajectories / seeds differ
    assert not np.array_equal(pkg.gen_layer(123, 5, 0, n, p)[1], pkg.gen_layer(123, 4, 0, n, p)[1])
    # the gate sample is Haar-like: mean |U_00|^2 = 1/4
    vals = [abs(pkg.gen_layer(9, 0, t, 4, 0.0)[1][0][0, 0]) ** 2 for t in range(400)]
    assert abs(np.mean(vals) - 0.25) < 0.03
