"""The plain-Python input generator of the CPU legs (oracle/gen_ref.py)
against the library's tn_gen_layer, bit for bit: the reference arm of the
benchmark must feed the oracle exactly the GPU arm's gates and uniforms
without loading the product library."""
import numpy as np
import pytest

from oracle import gen_ref


@pytest.mark.parametrize("n,p,seed,traj", [(64, 0.05, 20261203, 0), (64, 0.3, 20261203, 7), (17, 0.5, 3, 123456789)])
def test_python_generator_matches_library_bit_for_bit(pkg, n, p, seed, traj):
    for t in (0, 1, 2, 15, 34):
        a = pkg.gen_layer(seed, traj, t, n, p)
        b = gen_ref.gen_layer(seed, traj, t, n, p)
        for x, y in zip(a, b):
            assert x.shape == y.shape
            assert np.array_equal(x.view(np.uint8) if x.dtype.kind == "c" else x,
                                  y.view(np.uint8) if y.dtype.kind == "c" else y), (t, x, y)


def test_python_haar_is_unitary_with_positive_r_diagonal():
    q = gen_ref.haar_u4(gen_ref.ginibre(1, 2, 3, 4))
    np.testing.assert_allclose(q.conj().T @ q, np.eye(4), atol=1e-14)
    r = q.conj().T @ gen_ref.ginibre(1, 2, 3, 4)
    assert np.all(np.diag(r).real > 0) and np.allclose(np.diag(r).imag, 0, atol=1e-13)
