"""Fixed gate matrices (gate.rs:606-909) and the circuit element types, on
the CPU: every matrix against an independent definition of the same gate."""
import math

import numpy as np
import pytest

from gates import CX, CXREV, CZ, H, xrot


def _g():
    from tensor_net_gb300 import gates
    return gates


def test_fixed_matrices_match_definitions(pkg):
    g = _g()
    np.testing.assert_allclose(g.make_h(), H, atol=1e-15)
    np.testing.assert_array_equal(g.make_cx(), CX)
    np.testing.assert_array_equal(g.make_cxrev(), CXREV)
    np.testing.assert_array_equal(g.make_cz(), CZ)
    np.testing.assert_array_equal(g.make_z(), np.diag([1, -1]))
    np.testing.assert_array_equal(g.make_s(), np.diag([1, 1j]))
    np.testing.assert_array_equal(g.make_sinv(), np.diag([1, -1j]))
    np.testing.assert_array_equal(g.make_swap()[[0, 1, 2, 3]][:, [0, 2, 1, 3]], np.eye(4))
    # gate.rs:649-658 defines X as the identity
    np.testing.assert_array_equal(g.make_x(), np.eye(2))


@pytest.mark.parametrize("a", [0.0, 0.3, 1.7, -2.2, math.pi])
def test_rotations(pkg, a):
    g = _g()
    # XRot carries the global phase e^{i a/2} relative to exp(-i a X / 2)
    np.testing.assert_allclose(g.make_xrot(a), np.exp(0.5j * a) * xrot(a), atol=1e-15)
    np.testing.assert_allclose(g.make_zrot(a), np.diag([1, np.exp(1j * a)]), atol=1e-15)


@pytest.mark.parametrize("abc", [(0.1, 0.2, 0.3), (1.3, -0.7, 2.9), (0.0, math.pi, 0.0)])
def test_euler_u_is_zxz_and_unitary(pkg, abc):
    g = _g()
    a, b, c = abc
    u = g.make_u(a, b, c)
    np.testing.assert_allclose(u, g.make_zrot(a) @ g.make_xrot(b) @ g.make_zrot(c), atol=1e-14)
    np.testing.assert_allclose(u @ u.conj().T, np.eye(2), atol=1e-14)


def test_gate_values_and_kinds(pkg):
    g = _g()
    G = g.Gate
    assert G.U(3, 0.1, 0.2, 0.3).is_q1() and not G.U(3, 0.1, 0.2, 0.3).is_q2()
    for q1 in (G.H(0), G.X(1), G.Z(2), G.S(3), G.SInv(4), G.XRot(5, 0.1), G.ZRot(6, 0.2)):
        assert q1.is_q1() and q1.into_matrix()[1].shape == (2, 2)
    for q2 in (G.CX(0), G.CXRev(1), G.CZ(2)):
        assert q2.is_q2() and q2.into_matrix()[1].shape == (4, 4)
    k, m = G.Haar2(4).into_matrix(np.random.default_rng(1))
    assert k == 4 and m.shape == (4, 4)
    np.testing.assert_allclose(m @ m.conj().T, np.eye(4), atol=1e-13)
    with pytest.raises(ValueError):
        G.Haar2(0).into_matrix()
    with pytest.raises(ValueError):
        g.Gate("XRot", 0)
    with pytest.raises(ValueError):
        g.Gate("Y", 0)


def test_uni_and_meas_values(pkg):
    g = _g()
    assert g.Uni.of_gate(g.Gate.H(2)).is_gate() and g.Uni.of_gate(g.Gate.H(2)).idx() == 2
    m = g.Uni.mat(3, np.eye(4))
    assert m.is_mat() and m == g.Uni.mat(3, np.eye(4)) and m != g.Uni.mat(3, 2 * np.eye(4))
    assert g.Meas.rand(1).is_rand() and g.Meas.proj(1, 1).is_proj()
    with pytest.raises(ValueError):
        g.Meas.proj(0, 2)
