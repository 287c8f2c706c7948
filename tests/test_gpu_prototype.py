"""The GPU path against outputs of the reference's own Python prototypes
(tests/golden/prototype.npz, from prototyping/schmidt_mps.py; the same
fixture holds the oracle in tests/test_prototype_golden.py), float64:

* ``tn_mps_from_vector`` against ``canonicalize`` on seeded states, n = 2..8:
  every bond's Schmidt values and the contracted state to 1e-12;
* ``tn_mps_apply_unitary2`` on a two-qubit state against ``apply_2q`` (exact
  for two qubits): the Schmidt values and the state after the gate.
"""
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "prototype.npz")


@pytest.mark.parametrize("n", range(2, 9))
def test_from_vector_matches_canonicalize(pkg, n):
    g = pkg.MPS.from_vector(G[f"schmidt_n{n}_psi"])
    for b in range(n - 1):
        ref = G[f"schmidt_n{n}_L{b}"]
        sg = g.svals(b)
        assert len(sg) == len(ref), (n, b, len(sg), len(ref))
        np.testing.assert_allclose(sg, ref, rtol=0, atol=1e-12)
    np.testing.assert_allclose(g.contract(), G[f"schmidt_n{n}_contract"], rtol=0, atol=1e-12)
    assert g.device_status() == 0


def test_two_qubit_gate_matches_apply_2q(pkg):
    for i in range(6):
        g = pkg.MPS.from_vector(G[f"gate2_{i}_psi"])
        g.apply_unitary2(0, G[f"gate2_{i}_u"])
        ref = G[f"gate2_{i}_L"]
        sg = g.svals(0)
        assert len(sg) == len(ref) == 2, (i, len(sg))
        np.testing.assert_allclose(sg, ref, rtol=0, atol=1e-12)
        np.testing.assert_allclose(g.contract(), G[f"gate2_{i}_contract"], rtol=0, atol=1e-12)
        assert g.device_status() == 0
