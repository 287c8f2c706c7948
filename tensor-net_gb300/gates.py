"""Fixed gates and circuit elements of tensor-net.

* ``Gate`` mirrors the enum of tensor-net/lib/gate.rs:25-57: one-qubit
  ``U(k, alpha, beta, gamma)``, ``H``, ``X``, ``Z``, ``S``, ``SInv``,
  ``XRot(k, angle)``, ``ZRot(k, angle)``; two-qubit ``CX``, ``CXRev``, ``CZ``,
  ``Haar2`` (``k`` is always the left qubit).  ``into_matrix`` follows
  gate.rs:226-262 and the ``make_*`` constructors gate.rs:606-909.
* ``Uni`` (circuit.rs:210-216) is either ``Uni.of_gate(Gate)`` or
  ``Uni.mat(k, matrix)`` (2x2 or 4x4).
* ``Meas`` (circuit.rs:345-348) is ``Meas.rand(k)`` or ``Meas.proj(k, outcome)``
  with ``Outcome`` 0 (``Zero``) or 1 (``One``) (circuit.rs:73-78).

The matrices are built on the host (they are 2x2 / 4x4 constants); applying
them runs through ``MPS.apply_unitary1`` / ``apply_unitary2`` on the GPU.

``make_x`` returns the 2x2 identity, as gate.rs:649-658 does: the reference's
``X`` gate (and ``XMAT``) is the identity matrix, and a drop-in keeps that.
``Haar2`` needs randomness, which the caller supplies (a numpy ``Generator``
or a 4x4 complex Ginibre sample); the reference's ChaCha/statrs stream is not
reproduced.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .inputs import haar_u4

ZERO, ONE = 0, 1


def _cis(x: float) -> complex:
    return complex(math.cos(x), math.sin(x))


def make_u(alpha: float, beta: float, gamma: float) -> np.ndarray:
    """gate.rs:606-624: Euler-angle unitary, e^{i b/2} [[c, -i e^{i g} s], [-i e^{i a} s, e^{i(a+g)} c]]
    with c, s = cos(b/2), sin(b/2) -- equal to ZRot(alpha) . XRot(beta) . ZRot(gamma)."""
    b2 = beta / 2.0
    pre = _cis(b2)
    on0 = math.cos(b2)
    on1 = _cis(alpha + gamma) * on0
    off = math.sin(b2)
    off0 = -1j * _cis(gamma) * off
    off1 = -1j * _cis(alpha) * off
    return np.array([[pre * on0, pre * off0], [pre * off1, pre * on1]], dtype=np.complex128)


def make_h() -> np.ndarray:
    """gate.rs:630-640."""
    h = math.sqrt(0.5)
    return np.array([[h, h], [h, -h]], dtype=np.complex128)


def make_x() -> np.ndarray:
    """gate.rs:649-658: the identity (the reference's definition of its X gate)."""
    return np.eye(2, dtype=np.complex128)


def make_z() -> np.ndarray:
    """gate.rs:667-676."""
    return np.diag([1.0, -1.0]).astype(np.complex128)


def make_s() -> np.ndarray:
    """gate.rs:685-694."""
    return np.diag([1.0, 1j]).astype(np.complex128)


def make_sinv() -> np.ndarray:
    """gate.rs:703-712."""
    return np.diag([1.0, -1j]).astype(np.complex128)


def make_xrot(angle: float) -> np.ndarray:
    """gate.rs:718-731: e^{i a/2} [[cos(a/2), -i sin(a/2)], [-i sin(a/2), cos(a/2)]]."""
    a2 = angle / 2.0
    pre = _cis(a2)
    on = math.cos(a2)
    off = -1j * math.sin(a2)
    return np.array([[pre * on, pre * off], [pre * off, pre * on]], dtype=np.complex128)


def make_zrot(angle: float) -> np.ndarray:
    """gate.rs:734-744: diag(1, e^{i angle})."""
    return np.array([[1.0, 0.0], [0.0, _cis(angle)]], dtype=np.complex128)


def _perm4(cols) -> np.ndarray:
    m = np.zeros((4, 4), dtype=np.complex128)
    for r, c in enumerate(cols):
        m[r, c] = 1.0
    return m


def make_cx() -> np.ndarray:
    """gate.rs:750-761: control = left qubit (the high bit of the fused index)."""
    return _perm4([0, 1, 3, 2])


def make_cxrev() -> np.ndarray:
    """gate.rs:785-796: control = right qubit."""
    return _perm4([0, 3, 2, 1])


def make_cz() -> np.ndarray:
    """gate.rs:821-832."""
    return np.diag([1.0, 1.0, 1.0, -1.0]).astype(np.complex128)


def make_swap() -> np.ndarray:
    """gate.rs:856-867."""
    return _perm4([0, 2, 1, 3])


def haar(rng=None, z=None) -> np.ndarray:
    """``gate::haar(2, rng)`` (gate.rs:888-909): QR of a 4x4 complex Ginibre
    matrix, columns rephased so that R has a positive real diagonal.  ``z``
    is the Ginibre sample; without it one is drawn from ``rng`` (a numpy
    Generator; real then imaginary part of each entry, row-major)."""
    if z is None:
        if rng is None:
            raise ValueError("Haar2 needs a random generator or a Ginibre sample")
        x = rng.standard_normal(32).reshape(4, 4, 2)
        z = x[..., 0] + 1j * x[..., 1]
    return haar_u4(z)


Q1_KINDS = ("U", "H", "X", "Z", "S", "SInv", "XRot", "ZRot")
Q2_KINDS = ("CX", "CXRev", "CZ", "Haar2")
_NPARAMS = {"U": 3, "XRot": 1, "ZRot": 1}


@dataclass(frozen=True)
class Gate:
    """One gate of gate.rs:25-57: ``kind`` names the variant, ``k`` is the
    (left) qubit, ``params`` the angles of ``U`` / ``XRot`` / ``ZRot``."""

    kind: str
    k: int
    params: tuple = ()

    def __post_init__(self):
        if self.kind not in Q1_KINDS and self.kind not in Q2_KINDS:
            raise ValueError(f"unknown gate kind {self.kind!r}")
        if len(self.params) != _NPARAMS.get(self.kind, 0):
            raise ValueError(f"{self.kind} takes {_NPARAMS.get(self.kind, 0)} angle(s)")

    # constructors named like the reference's variants
    @staticmethod
    def U(k, alpha, beta, gamma):
        return Gate("U", int(k), (float(alpha), float(beta), float(gamma)))

    @staticmethod
    def H(k):
        return Gate("H", int(k))

    @staticmethod
    def X(k):
        return Gate("X", int(k))

    @staticmethod
    def Z(k):
        return Gate("Z", int(k))

    @staticmethod
    def S(k):
        return Gate("S", int(k))

    @staticmethod
    def SInv(k):
        return Gate("SInv", int(k))

    @staticmethod
    def XRot(k, angle):
        return Gate("XRot", int(k), (float(angle),))

    @staticmethod
    def ZRot(k, angle):
        return Gate("ZRot", int(k), (float(angle),))

    @staticmethod
    def CX(k):
        return Gate("CX", int(k))

    @staticmethod
    def CXRev(k):
        return Gate("CXRev", int(k))

    @staticmethod
    def CZ(k):
        return Gate("CZ", int(k))

    @staticmethod
    def Haar2(k):
        return Gate("Haar2", int(k))

    def idx(self) -> int:
        return self.k

    def is_q1(self) -> bool:
        return self.kind in Q1_KINDS

    def is_q2(self) -> bool:
        return self.kind in Q2_KINDS

    def into_matrix(self, rng=None, z=None):
        """``(k, matrix)`` (gate.rs:226-262); ``Haar2`` draws from ``rng`` (or uses ``z``)."""
        kd, p = self.kind, self.params
        if kd == "U":
            m = make_u(*p)
        elif kd == "H":
            m = make_h()
        elif kd == "X":
            m = make_x()
        elif kd == "Z":
            m = make_z()
        elif kd == "S":
            m = make_s()
        elif kd == "SInv":
            m = make_sinv()
        elif kd == "XRot":
            m = make_xrot(*p)
        elif kd == "ZRot":
            m = make_zrot(*p)
        elif kd == "CX":
            m = make_cx()
        elif kd == "CXRev":
            m = make_cxrev()
        elif kd == "CZ":
            m = make_cz()
        else:
            m = haar(rng, z)
        return self.k, m


@dataclass(frozen=True)
class Uni:
    """``Uni`` (circuit.rs:210-216): ``gate`` is a ``Gate`` or ``None``; for a
    ``Mat`` the qubit ``k`` and the matrix (2x2 or 4x4, assumed unitary)."""

    gate: Gate | None = None
    k: int = 0
    matrix: np.ndarray | None = None

    @staticmethod
    def of_gate(g: Gate) -> "Uni":
        return Uni(gate=g, k=g.k)

    @staticmethod
    def mat(k: int, m) -> "Uni":
        return Uni(gate=None, k=int(k), matrix=np.asarray(m, dtype=np.complex128))

    def is_gate(self) -> bool:
        return self.gate is not None

    def is_mat(self) -> bool:
        return self.gate is None

    def idx(self) -> int:
        return self.k

    def __eq__(self, other):
        if not isinstance(other, Uni):
            return NotImplemented
        if self.is_gate() or other.is_gate():
            return self.gate == other.gate
        return self.k == other.k and self.matrix.shape == other.matrix.shape and \
            bool(np.array_equal(self.matrix, other.matrix))

    def __hash__(self):
        return hash((self.gate, self.k))


@dataclass(frozen=True, order=True)
class Meas:
    """``Meas`` (circuit.rs:345-348): ``Rand(k)`` when ``outcome`` is None,
    else ``Proj(k, outcome)``."""

    k: int
    outcome: int | None = None

    @staticmethod
    def rand(k: int) -> "Meas":
        return Meas(int(k), None)

    @staticmethod
    def proj(k: int, outcome: int) -> "Meas":
        if outcome not in (ZERO, ONE):
            raise ValueError("outcome must be 0 (Zero) or 1 (One)")
        return Meas(int(k), int(outcome))

    def is_rand(self) -> bool:
        return self.outcome is None

    def is_proj(self) -> bool:
        return self.outcome is not None

    def idx(self) -> int:
        return self.k
