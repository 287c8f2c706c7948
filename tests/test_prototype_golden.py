"""The oracle against outputs of the reference's own Python prototypes.

tests/golden/prototype.npz was written by tests/golden/make_prototype_golden.py
from the reference tree's prototyping/haar-unitary.py (``random_haar``) and
prototyping/schmidt_mps.py (``canonicalize``, ``contract``, ``apply_1q``,
``apply_2q``, ``project``) and prototyping/entropy.py (``trace_qubit``,
``entropy_log``), run on seeded inputs.  These are the only parts of the
reference that run here (the library is Rust), so they pin these pieces of
the oracle to code the reference ships:

* the Haar recipe of ``gate::haar`` (gate.rs:888-909): the oracle's numpy
  form and the restatement of the C++ input generator's Gram-Schmidt form
  give the prototype's unitary from the same Ginibre matrix;
* ``factorize`` / ``from_vector`` (mps.rs:448-550): the Schmidt values of
  every bond and the contracted state of seeded states, n = 2..8;
* a two-qubit gate on a two-qubit state (the one case where the prototype's
  ``apply_2q``, which leaves the outer Lambdas out of theta, is exact): the
  Schmidt values and the state after ``apply_unitary2``;
* ``apply_unitary1`` (mps.rs:1298-1314) against ``apply_1q``: the state;
* ``entropy_vn`` against ``entropy_log`` of the reduced density matrix
  (prototyping/entropy.py's ``trace_qubit``) on every bond;
* ``local_prob`` + ``project`` + the refactor sweep of
  ``measure_postsel_prob`` (mps.rs:1079-1134, 1453-1465, 1501-1510) against
  ``project`` where the prototype's contraction spans the whole chain (n = 2,
  the middle site of n = 3): probability and Schmidt values, and for n = 2
  the state (the prototype's middle-site branch leaves Gammas that do not
  contract back to the projected state; its Schmidt values are right).  The
  prototype keeps every singular value above 0, so values at rounding level
  (a product state's second one) are compared as zero.
"""
import pathlib

import numpy as np
import pytest

from oracle import gen_ref, mps_ref

G = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "prototype.npz")


def test_haar_recipe_matches_the_prototype():
    assert len(G["haar_z"]) == 8
    for z, u in zip(G["haar_z"], G["haar_u"]):
        np.testing.assert_allclose(mps_ref.haar_from_ginibre(z), u, rtol=0, atol=1e-13)
        np.testing.assert_allclose(gen_ref.haar_u4(z), u, rtol=0, atol=1e-13)
        np.testing.assert_allclose(u.conj().T @ u, np.eye(4), rtol=0, atol=1e-13)


@pytest.mark.parametrize("n", range(2, 9))
def test_factorize_matches_canonicalize(n):
    psi = G[f"schmidt_n{n}_psi"]
    m = mps_ref.from_vector(psi)
    for b in range(n - 1):
        ref = G[f"schmidt_n{n}_L{b}"]
        assert len(m.svals[b]) == len(ref) == min(2 ** (b + 1), 2 ** (n - 1 - b)), (n, b)
        np.testing.assert_allclose(m.svals[b], ref, rtol=1e-12, atol=1e-14)
    # the prototype's contraction of its own MPS returns its input, and so does the oracle's
    np.testing.assert_allclose(G[f"schmidt_n{n}_contract"], psi, rtol=0, atol=1e-12)
    np.testing.assert_allclose(m.contract(), psi, rtol=0, atol=1e-12)


def test_two_qubit_gate_matches_apply_2q():
    for i in range(6):
        psi, u = G[f"gate2_{i}_psi"], G[f"gate2_{i}_u"]
        m = mps_ref.from_vector(psi)
        m.apply_unitary2(0, u)
        ref = G[f"gate2_{i}_L"]
        assert len(m.svals[0]) == len(ref) == 2
        np.testing.assert_allclose(m.svals[0], ref, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(G[f"gate2_{i}_contract"], u @ psi, rtol=0, atol=1e-12)
        np.testing.assert_allclose(m.contract(), u @ psi, rtol=0, atol=1e-12)


def test_one_qubit_gate_matches_apply_1q():
    for i in range(4):
        n, k = (int(x) for x in G[f"gate1_{i}_nk"])
        psi, u = G[f"gate1_{i}_psi"], G[f"gate1_{i}_u"]
        m = mps_ref.from_vector(psi)
        m.apply_unitary1(k, u)
        want = np.einsum("ab,lbr->lar", u, psi.reshape(2 ** k, 2, 2 ** (n - 1 - k))).reshape(-1)
        np.testing.assert_allclose(G[f"gate1_{i}_contract"], want, rtol=0, atol=1e-12)
        np.testing.assert_allclose(m.contract(), G[f"gate1_{i}_contract"], rtol=0, atol=1e-12)


def _above(s, floor=1e-10):
    s = np.asarray(s)
    assert np.all(s[s <= floor] < 1e-12), s  # below the floor only rounding noise
    return s[s > floor]


def test_projection_matches_project():
    for i in range(6):
        n, k, p = (int(x) for x in G[f"proj_{i}_nkp"])
        psi = G[f"proj_{i}_psi"]
        # the projected, renormalised state and its probability, from the vector itself
        v = psi.reshape(2 ** k, 2, 2 ** (n - 1 - k)).copy()
        v[:, 1 - p, :] = 0.0
        v = v.reshape(-1)
        prob = float(np.vdot(v, v).real)
        want = v / np.sqrt(prob)
        if n == 2:
            # (the prototype's middle-site branch returns the right Schmidt values but
            # Gammas that do not contract back to the projected state, so its state is
            # compared only for n = 2)
            np.testing.assert_allclose(G[f"proj_{i}_contract"], want, rtol=0, atol=1e-12)
        m = mps_ref.from_vector(psi)
        assert abs(m.local_prob(k, p) - prob) < 1e-13
        got = m.measure_postsel_prob(k, p)
        assert abs(got - prob) < 1e-13
        np.testing.assert_allclose(m.contract(), want, rtol=0, atol=1e-12)
        for b in range(n - 1):
            ref = _above(G[f"proj_{i}_L{b}"])
            np.testing.assert_allclose(_above(m.svals[b]), ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("n", [4, 6, 8])
def test_entropy_matches_the_reduced_density_matrix(n):
    """entropy_vn (mps.rs:1251-1261) on every bond against -tr(rho log rho) of
    the reduced density matrix, by the reference's prototyping/entropy.py."""
    m = mps_ref.from_vector(G[f"schmidt_n{n}_psi"])
    got = np.array([m.entropy_vn(b) for b in range(n - 1)])
    np.testing.assert_allclose(got, G[f"entropy_n{n}"], rtol=0, atol=1e-12)
