"""The oracle against outputs of the reference's own Python prototypes.

tests/golden/prototype.npz was written by tests/golden/make_prototype_golden.py
from the reference tree's prototyping/haar-unitary.py (``random_haar``) and
prototyping/schmidt_mps.py (``canonicalize``, ``contract``, ``apply_2q``),
run on seeded inputs.  These are the only parts of the reference that run
here (the library is Rust), so they pin three pieces of the oracle to code
the reference ships:

* the Haar recipe of ``gate::haar`` (gate.rs:888-909): the oracle's numpy
  form and the restatement of the C++ input generator's Gram-Schmidt form
  give the prototype's unitary from the same Ginibre matrix;
* ``factorize`` / ``from_vector`` (mps.rs:448-550): the Schmidt values of
  every bond and the contracted state of seeded states, n = 2..8;
* a two-qubit gate on a two-qubit state (the one case where the prototype's
  ``apply_2q``, which leaves the outer Lambdas out of theta, is exact): the
  Schmidt values and the state after ``apply_unitary2``.
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
