"""FP64 CPU oracle for the Schmidt-form (Gamma-Lambda) MPS trajectory path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path may import, call or
execute this module; only ``tests/`` (including the golden-fixture generator),
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py``
(``cpu_baseline``, ``--impl reference``, the single-core timing of
``--workload plain``) use it, and only as the checker or the timed CPU
baseline.

This is a step-by-step restatement of whooie/tensor-net's ``MPS<Q, C64>``
(``tensor-net/lib/mps.rs``), its Haar sampler (``tensor-net/lib/gate.rs``) and
its brickwork circuit layer (``tensor-net/lib/circuit.rs``), in complex128 with
numpy.  Every function names the reference lines it follows.

Parity pin.  The reference is Rust and cannot be built here (no cargo/rustc, and
its dependencies need the network), so it cannot be run to produce golden
outputs.  The one piece of arithmetic it delegates to a third party is the SVD:
``SVDInto::svd_into(true, true)`` from ndarray-linalg 0.16.0 / lax 0.16.0 over
openblas-src 0.10.11, i.e. LAPACK ``zgesvd`` (mps.rs:299).  The restatement
calls the same LAPACK driver through ``scipy.linalg.svd(...,
lapack_driver="gesvd")``.  The oracle is pinned by the reference's own
known-answer programs (``workspace/src/rotation_testing.rs``,
``density_mat_testing.rs``, ``testing.rs``, ``state.rs``, the ``mps.rs:43-95``
doc example), restated as tests in ``tests/test_oracle_known_answers.py``, and
by dense state-vector cross-checks.  No reference-produced vectors exist for
the LAPACK boundary itself; results compared there are gauge invariant
(Schmidt values, probabilities, outcomes, entropies).

Randomness.  The reference draws from ``rand::Rng`` inside ``sample_state``
(mps.rs:1433) and ``uniform_meas`` (circuit.rs:580-584).  The oracle (and the
GPU library) instead take caller-supplied uniforms: ``us[j]`` is the draw used
for the j-th measured site in ascending site order, which is the order the
reference consumes its RNG in ``apply_meas_prob_layer`` (mps.rs:2224-2245).

Truncation.  ``BondDim`` (mps.rs:157-166) is ``Const(r)`` or ``Cutoff(eps)``;
``Trunc.both(r, eps)`` is the combined rule used by the benchmark workloads:
``rank = max(1, min(r, #{leading s_j normal and > |eps|}))``.  It equals
``Const(r)`` at ``eps = f64::EPSILON`` and ``Cutoff(eps)`` at ``r = inf``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import scipy.linalg

F64_EPS = float(np.finfo(np.float64).eps)

MODE_NONE, MODE_CONST, MODE_CUTOFF, MODE_BOTH = 0, 1, 2, 3


@dataclass(frozen=True)
class Trunc:
    """``Option<BondDim<f64>>`` (mps.rs:157-166) plus the combined rule."""

    mode: int = MODE_NONE
    chi_max: int = 0
    cutoff: float = 0.0

    @staticmethod
    def none() -> "Trunc":
        return Trunc(MODE_NONE, 0, 0.0)

    @staticmethod
    def const(r: int) -> "Trunc":
        return Trunc(MODE_CONST, int(r), 0.0)

    @staticmethod
    def cut(eps: float) -> "Trunc":
        return Trunc(MODE_CUTOFF, 0, float(eps))

    @staticmethod
    def both(r: int, eps: float) -> "Trunc":
        return Trunc(MODE_BOTH, int(r), float(eps))


def _leading_count(s: np.ndarray, eps: float) -> int:
    """``s.iter().take_while(|sj| sj.is_normal() && **sj > eps).count()``."""
    n = 0
    for sj in s:
        # f64::is_normal: finite, non-zero, not subnormal.
        if not (math.isfinite(sj) and sj != 0.0 and abs(sj) >= np.finfo(np.float64).tiny):
            break
        if not sj > eps:
            break
        n += 1
    return n


def rank_rule(s: np.ndarray, trunc: Trunc) -> int:
    """Rank selection of ``process_svd`` (mps.rs:250-274), on normalised s."""
    if trunc.mode == MODE_CONST:
        return min(max(trunc.chi_max, 1), _leading_count(s, F64_EPS))
    if trunc.mode == MODE_CUTOFF:
        return max(_leading_count(s, abs(trunc.cutoff)), 1)
    if trunc.mode == MODE_BOTH:
        return max(1, min(trunc.chi_max, _leading_count(s, abs(trunc.cutoff))))
    return max(_leading_count(s, F64_EPS), 1)


def process_svd(u, s, vh, trunc: Trunc):
    """``process_svd`` (mps.rs:236-293).

    Returns ``(u[:, :rank], s_kept_renormalised, q, rank)`` where row j of q is
    ``vh[j] * s_j / ||s||`` (the right Schmidt vector scaled by its Schmidt
    value before the second renormalisation), exactly as the reference's
    ``q_j *= s_j * renorm`` leaves it.
    """
    norm = math.sqrt(float(np.sum(s * s)))
    s = s / norm
    rank = rank_rule(s, trunc)
    s = s[:rank]
    norm2 = math.sqrt(float(np.sum(s * s)))
    s = s / norm2
    q = vh[:rank, :] * (s * norm2)[:, None]
    return u[:, :rank], s, q, rank


def local_decomp(theta: np.ndarray, trunc: Trunc):
    """``SchmidtDecomp::local_decomp`` (mps.rs:295-303): full SVD by LAPACK
    gesvd (the driver ndarray-linalg's ``svd_into`` calls), then process_svd."""
    u, s, vh = scipy.linalg.svd(theta, full_matrices=True, lapack_driver="gesvd",
                                check_finite=False)
    return process_svd(u, s, vh, trunc)


def haar_from_ginibre(z: np.ndarray) -> np.ndarray:
    """``gate::haar`` (gate.rs:888-909) given the Ginibre sample ``z``.

    QR of z, then column j of Q divided by ``r_jj / |r_jj|`` (gate.rs:902-907).
    The result is the unique Q whose R has a positive real diagonal, so any
    correct QR gives the same matrix.
    """
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q / (d / np.abs(d))[None, :]


def tile_q2(n: int, offs: bool):
    """``TileQ2::new(nqubits, offs)`` (circuit.rs:523-531)."""
    return list(range(int(bool(offs)), n - 1, 2))


class MPS:
    """``MPS<Q, C64>`` (mps.rs:339-356) on qubits.

    ``data[k]`` has shape (chi_{k-1}, 2, chi_k); ``svals[k]`` is Lambda on bond k
    (length chi_k, n-1 bonds).
    """

    def __init__(self, n: int, trunc: Trunc | None = None):
        """``MPS::new`` / ``MPS::new_qubits`` (mps.rs:370-391, 2033-2039)."""
        if n < 1:
            raise ValueError("EmptySystem")
        self.n = n
        self.trunc = trunc if trunc is not None else Trunc.none()
        self.data = []
        for _ in range(n):
            g = np.zeros((1, 2, 1), dtype=np.complex128)
            g[0, 0, 0] = 1.0
            self.data.append(g)
        self.svals = [np.ones(1, dtype=np.float64) for _ in range(n - 1)]

    def copy(self) -> "MPS":
        m = MPS.__new__(MPS)
        m.n, m.trunc = self.n, self.trunc
        m.data = [g.copy() for g in self.data]
        m.svals = [s.copy() for s in self.svals]
        return m

    # -- contraction -------------------------------------------------------
    def contract_local2(self, k: int) -> np.ndarray:
        """``contract_local2`` (mps.rs:732-754) via ``do_contract2``
        (mps.rs:628-651): theta[(v s1), (s2 w)] with Lambda_{k-1} on rows and
        Lambda_{k+1} on columns (omitted at the chain ends)."""
        l, r = self.data[k], self.data[k + 1]
        cl, cr = l.shape[0], r.shape[2]
        lm = l.reshape(cl * 2, -1)
        rm = (r.reshape(r.shape[0], 2 * cr) * self.svals[k][:, None])
        q = (lm @ rm).reshape(cl, 2, 2, cr)
        if k != 0:
            q = q * self.svals[k - 1][:, None, None, None]
        if k != self.n - 2:
            q = q * self.svals[k + 1][None, None, None, :]
        return q.reshape(cl * 2, 2 * cr)

    def contract(self) -> np.ndarray:
        """``contract`` (mps.rs:794-798): the dense state vector, s_0 most
        significant.  Sequential rather than the reference's binary split
        (mps.rs:676-696); the same product."""
        psi = self.data[0].reshape(2, -1)
        for k in range(1, self.n):
            g = self.data[k]
            psi = (psi * self.svals[k - 1][None, :]) @ g.reshape(g.shape[0], -1)
            psi = psi.reshape(-1, g.shape[2])
        return psi.reshape(-1)

    # -- local (re)factorisation -------------------------------------------
    def _install(self, k: int, u, s, q, rank: int):
        """Gamma rebuild shared by ``local_refactor`` (mps.rs:856-879) and
        ``apply_unitary2`` (mps.rs:1357-1385)."""
        cl = self.data[k].shape[0]
        cr = self.data[k + 1].shape[2]
        gk = u.reshape(cl, 2, rank).copy()
        if k != 0:
            gk /= self.svals[k - 1][:, None, None]
        gk1 = q.reshape(rank, 2, cr).copy()
        gk1 /= s[:, None, None]
        if k != self.n - 2:
            gk1 /= self.svals[k + 1][None, None, :]
        self.data[k] = gk
        self.svals[k] = s
        self.data[k + 1] = gk1
        self.local_renormalize(k)
        self.local_renormalize(k + 1)

    def local_refactor(self, k: int):
        """``local_refactor`` (mps.rs:846-880)."""
        theta = self.contract_local2(k)
        u, s, q, rank = local_decomp(theta, self.trunc)
        self._install(k, u, s, q, rank)

    def refactor_sweep(self):
        """``refactor_sweep`` (mps.rs:894-897)."""
        for k in range(0, self.n - 1):
            self.local_refactor(k)
        for k in range(self.n - 3, -1, -1):
            self.local_refactor(k)

    # -- unitaries -----------------------------------------------------------
    def apply_unitary1(self, k: int, op: np.ndarray):
        """``apply_unitary1`` (mps.rs:1298-1314)."""
        if k >= self.n:
            return
        op = np.asarray(op, dtype=np.complex128)
        if op.shape != (2, 2):
            raise ValueError("OperatorIncompatibleShape")
        self.data[k] = np.einsum("ab,vbu->vau", op, self.data[k])

    def apply_unitary2(self, k: int, op: np.ndarray):
        """``apply_unitary2`` (mps.rs:1332-1387)."""
        if self.n == 1 or k >= self.n - 1:
            return
        op = np.asarray(op, dtype=np.complex128)
        if op.shape != (4, 4):
            raise ValueError("OperatorIncompatibleShape")
        cl = self.data[k].shape[0]
        cr = self.data[k + 1].shape[2]
        q = self.contract_local2(k).reshape(cl, 2, 2, cr).reshape(cl, 4, cr)
        q = np.einsum("ab,vbw->vaw", op, q)
        u, s, qq, rank = local_decomp(q.reshape(cl * 2, 2 * cr), self.trunc)
        self._install(k, u, s, qq, rank)

    # -- probabilities and norms ---------------------------------------------
    def _lam_left(self, k):
        return self.svals[k - 1] if k > 0 else np.ones(1)

    def _lam_right(self, k):
        return self.svals[k] if k < self.n - 1 else np.ones(1)

    def local_probs(self, k: int) -> np.ndarray:
        """``local_probs`` (mps.rs:1079-1134); all four branches reduce to
        sum_{v,u} L_{k-1}[v]^2 |G_k[v,s,u]|^2 L_k[u]^2 with the missing
        Lambda taken as [1]."""
        g = self.data[k]
        if self.n == 1:
            return (np.abs(g.reshape(-1)) ** 2)
        w = np.abs(g) ** 2
        w = w * (self._lam_left(k) ** 2)[:, None, None]
        w = w * (self._lam_right(k) ** 2)[None, None, :]
        return w.sum(axis=(0, 2))

    def local_prob(self, k: int, p: int) -> float:
        """``local_prob`` (mps.rs:1027-1066)."""
        return float(self.local_probs(k)[p])

    def probs(self, k: int):
        """``probs`` (mps.rs:1071-1076)."""
        if k >= self.n:
            return None
        return self.local_probs(k)

    def local_norm(self, k: int) -> float:
        """``local_norm`` (mps.rs:1147-1201): sqrt of the Lambda-weighted
        squared norm of G_k (real; the reference's complex sqrt of a sum of
        conj(g)*g with zero imaginary part)."""
        g = self.data[k]
        w = np.abs(g) ** 2
        w = w * (self._lam_left(k) ** 2)[:, None, None]
        w = w * (self._lam_right(k) ** 2)[None, None, :]
        return math.sqrt(float(w.sum()))

    def local_renormalize(self, k: int):
        """``local_renormalize`` (mps.rs:1206-1209)."""
        self.data[k] = self.data[k] / self.local_norm(k)

    # -- measurement -----------------------------------------------------------
    def sample_state(self, k: int, u: float):
        """``sample_state`` (mps.rs:1427-1447) with ``r = u`` (the draw the
        reference takes before computing the probabilities).  The first s with
        ``u < cumsum(p)_s``; the reference's ``unwrap`` would panic if none, the
        restatement takes the last outcome then."""
        probs = self.local_probs(k)
        cu = 0.0
        for j, pr in enumerate(probs):
            cu += pr
            if u < cu:
                return j, float(probs[j])
        j = len(probs) - 1
        return j, float(probs[j])

    def project(self, k: int, p: int, renorm: float):
        """``project`` (mps.rs:1453-1465)."""
        g = self.data[k].copy()
        for j in range(g.shape[1]):
            if j == p:
                g[:, j, :] /= renorm
            else:
                g[:, j, :] = 0.0
        self.data[k] = g

    def measure_prob(self, k: int, u: float):
        """``measure_prob`` (mps.rs:1479-1489)."""
        if k >= self.n:
            return None
        p, prob = self.sample_state(k, u)
        self.project(k, p, math.sqrt(prob))
        self.refactor_sweep()
        return p, prob

    def measure(self, k: int, u: float):
        """``measure`` (mps.rs:1471-1477)."""
        r = self.measure_prob(k, u)
        return None if r is None else r[0]

    def measure_postsel_prob(self, k: int, p: int):
        """``measure_postsel_prob`` (mps.rs:1501-1510)."""
        if k >= self.n or p >= 2:
            return None
        prob = self.local_prob(k, p)
        self.project(k, p, math.sqrt(prob))
        self.refactor_sweep()
        return prob

    def apply_meas_prob_layer(self, ks, us=None, posts=None):
        """``apply_meas_prob_layer`` (mps.rs:2206-2252).

        ``ks``: target sites (any order, duplicates allowed).  ``us[j]``: the
        uniform for the j-th target after filter/sort/dedup (``Meas::Rand``).
        ``posts[j]`` (optional, overrides ``us[j]``): a post-selected outcome
        for that target (``Meas::Proj``, mps.rs:2236-2242); ``None`` or a
        negative entry samples that target (``Meas::Rand``).  Returns a list of
        ``(k, outcome, prob)``.
        """
        targets = sorted(set(int(k) for k in ks if 0 <= int(k) < self.n))
        if not targets:
            return []
        last = None
        res = []
        for j, k in enumerate(targets):
            if last is not None:
                for b in range(last, k):
                    self.local_refactor(b)
            if posts is not None and posts[j] is not None and int(posts[j]) >= 0:
                p = int(posts[j])
                prob = self.local_prob(k, p)
            else:
                p, prob = self.sample_state(k, float(us[j]))
            self.project(k, p, math.sqrt(prob))
            res.append((k, p, prob))
            last = k
        for b in range(last, self.n - 1):
            self.local_refactor(b)
        for b in range(self.n - 3, -1, -1):
            self.local_refactor(b)
        return res

    # -- entropies / bonds ---------------------------------------------------
    def entropy_vn(self, b: int):
        """``entropy_vn`` (mps.rs:1251-1261)."""
        if not (0 <= b < self.n - 1):
            return None
        s2 = self.svals[b] ** 2
        return float(np.sum(-s2 * np.log(s2)))

    def entropy_ry_schmidt(self, a: float, b: int):
        """``entropy_ry_schmidt`` (mps.rs:1268-1282)."""
        if a == 1.0:
            return self.entropy_vn(b)
        if not (0 <= b < self.n - 1):
            return None
        s2 = self.svals[b] ** 2
        return float(np.log(np.sum(s2 ** a)) / (1.0 - a))

    def bond_dim(self, b: int):
        """``bond_dim`` (mps.rs:1243-1245)."""
        return len(self.svals[b]) if 0 <= b < self.n - 1 else None

    def max_bond_dim(self):
        """``max_bond_dim`` (mps.rs:1224-1226)."""
        return max((len(s) for s in self.svals), default=None)


def from_vector(state, trunc: Trunc | None = None) -> MPS:
    """``MPS::from_vector`` over qubits (mps.rs:517-550) with ``factorize``
    (mps.rs:448-505): normalise, then left to right reshape the remainder to
    (2 chi_{k-1}, rest), SVD + ``process_svd``, Gamma_k = U[:, :rank] reshaped
    (chi_{k-1}, 2, rank) divided by Lambda_{k-1} on its first axis, carry q on;
    the last Gamma is q reshaped (chi_{n-2}, 2, 1) divided by Lambda_{n-2}."""
    psi = np.asarray(state, dtype=np.complex128).reshape(-1)
    n = int(round(math.log2(psi.size))) if psi.size else 0
    if psi.size == 0:
        raise ValueError("EmptySystem")
    if (1 << n) != psi.size:
        raise ValueError("StateIncompatibleShape")
    psi = psi / math.sqrt(float(np.sum(np.abs(psi) ** 2)))
    m = MPS(n, trunc)
    if n == 1:
        m.data[0] = psi.reshape(1, 2, 1).copy()
        return m
    tr = trunc if trunc is not None else Trunc.none()
    q = psi.reshape(1, -1)
    udim = 1
    for k in range(n - 1):
        q = q.reshape(udim * 2, -1)
        u, s, q, rank = local_decomp(q, tr)
        g = u.reshape(udim, 2, rank).copy()
        if k > 0:
            g /= m.svals[k - 1][:, None, None]
        m.data[k] = g
        m.svals[k] = s
        udim = rank
    g = q.reshape(udim, 2, 1).copy()
    g /= m.svals[n - 2][:, None, None]
    m.data[n - 1] = g
    return m


def apply_bilayer(mps: MPS, gate_ks, gates, meas_ks, us):
    """``circuit::apply_bilayer`` (circuit.rs:624-659) with ``Uni::Mat`` gates
    (``apply_uni_rng`` -> ``apply_unitary2``, mps.rs:2110-2126) followed by one
    ``apply_meas_prob_layer``.  Returns the (k, outcome, prob) list."""
    for k, op in zip(gate_ks, gates):
        mps.apply_unitary2(int(k), op)
    return mps.apply_meas_prob_layer(meas_ks, us)


def run_trajectory(n, trunc, layers, entropy_bond=None):
    """Run a list of layers ``(gate_ks, gates, meas_ks, us)`` from |0...0>
    and return per-layer half-chain entropies and the measurement records
    (the trajectory driver of workspace/src/haar_coev_probs.rs:34-80 with the
    record kept, entropy read as in circuit_old.rs:405-434)."""
    mps = MPS(n, trunc)
    b = (n // 2 - 1) if entropy_bond is None else entropy_bond
    ents, recs = [], []
    for (gk, g, mk, us) in layers:
        recs.append(apply_bilayer(mps, gk, g, mk, us))
        ents.append(mps.entropy_vn(b))
    return mps, np.array(ents), recs
