"""Fixed gate matrices used by the known-answer tests (the standard
definitions tensor-net uses in gate.rs: H, X-rotation, CX, CX reversed, CZ)."""
import numpy as np

H = np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2)
CX = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
CXREV = np.array([[1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0]], dtype=np.complex128)
CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)


def xrot(theta):
    """exp(-i theta X / 2)."""
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)


def dense_apply2(psi, n, k, op):
    """Apply a 4x4 op on qubits (k, k+1) of a dense state (qubit 0 most significant)."""
    t = psi.reshape([2] * n)
    t = np.moveaxis(t, (k, k + 1), (0, 1)).reshape(4, -1)
    t = (op @ t).reshape([2, 2] + [2] * (n - 2))
    return np.moveaxis(t, (0, 1), (k, k + 1)).reshape(-1)


def dense_apply1(psi, n, k, op):
    t = psi.reshape([2] * n)
    t = np.moveaxis(t, k, 0).reshape(2, -1)
    t = (op @ t).reshape([2] + [2] * (n - 1))
    return np.moveaxis(t, 0, k).reshape(-1)


def dense_probs(psi, n, k):
    t = np.abs(psi.reshape([2] * n)) ** 2
    t = np.moveaxis(t, k, 0).reshape(2, -1)
    return t.sum(axis=1)


def dense_project(psi, n, k, p):
    t = psi.reshape([2] * n).copy()
    t = np.moveaxis(t, k, 0)
    t[1 - p] = 0
    t = np.moveaxis(t, 0, k).reshape(-1)
    return t / np.linalg.norm(t)


def dense_entropy(psi, n, b):
    m = psi.reshape(2 ** (b + 1), -1)
    s = np.linalg.svd(m, compute_uv=False)
    s2 = s[s > 1e-14] ** 2
    return float(-(s2 * np.log(s2)).sum())


def swap_gates():
    """SWAP as CX . CXRev . CX (workspace/src/testing.rs:19-24)."""
    return [CX, CXREV, CX]
