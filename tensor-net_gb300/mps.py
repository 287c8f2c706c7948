"""Host-side mirror of tensor-net's ``MPS<Q, C64>`` over the C ABI.

Method names, argument meaning and out-of-range behaviour follow
``tensor-net/lib/mps.rs``; the state lives on the GPU (``tn_mps`` handle).
Randomness is caller-supplied: every measurement takes the uniform the
reference would have drawn from its ``rng`` at that point.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

MODE_NONE, MODE_CONST, MODE_CUTOFF, MODE_BOTH = 0, 1, 2, 3
PRECISIONS = {"f64": 0, "mixed": 1, "df": 2}


@dataclass(frozen=True)
class Trunc:
    """``Option<BondDim<f64>>`` (mps.rs:157-166) plus the combined rule
    ``rank = max(1, min(chi_max, #{s_j > cutoff}))`` (``Trunc.both``)."""

    mode: int = MODE_NONE
    chi_max: int = 0
    cutoff: float = 0.0

    @staticmethod
    def none():
        return Trunc(MODE_NONE, 0, 0.0)

    @staticmethod
    def const(r: int):
        return Trunc(MODE_CONST, int(r), 0.0)

    @staticmethod
    def cut(eps: float):
        return Trunc(MODE_CUTOFF, 0, float(eps))

    @staticmethod
    def both(r: int, eps: float):
        return Trunc(MODE_BOTH, int(r), float(eps))

    def c(self) -> L.tn_trunc:
        return L.tn_trunc(int(self.mode), int(self.chi_max), float(self.cutoff))


def _as_op(op, d: int):
    a = np.ascontiguousarray(np.asarray(op, dtype=np.complex128))
    if a.ndim != 2:
        a = a.reshape(1, -1)
    return a.view(np.float64).reshape(-1).copy(), a.shape


class MPS:
    """GPU-resident Schmidt-form MPS of qubits (mps.rs:339-356)."""

    def __init__(self, n: int, trunc: Trunc | None = None, precision: str = "f64", chi_cap: int = 0,
                 _handle=None):
        self._lib = L.lib()
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            tr = C.byref(trunc.c()) if trunc is not None else None
            L.check(self._lib.tn_mps_new_qubits(int(n), tr, PRECISIONS[precision], int(chi_cap),
                                                C.byref(self._h)), "tn_mps_new_qubits")
        nn = L.u32()
        L.check(self._lib.tn_mps_n(self._h, C.byref(nn)), "tn_mps_n")
        self.n = int(nn.value)

    @classmethod
    def new_qubits(cls, n: int, trunc: Trunc | None = None, precision: str = "f64", chi_cap: int = 0):
        """``MPS::new_qubits`` (mps.rs:2033-2039)."""
        return cls(n, trunc, precision, chi_cap)

    @classmethod
    def from_vector(cls, state, trunc: Trunc | None = None, precision: str = "f64", chi_cap: int = 0):
        """``MPS::from_vector`` over qubits (mps.rs:517-550): normalise the
        2^n amplitudes (s_0 most significant) and factorise them on the GPU
        (``tn_mps_from_vector``); n <= 20."""
        a = np.ascontiguousarray(np.asarray(state, dtype=np.complex128).reshape(-1))
        n = max(int(a.size).bit_length() - 1, 0)
        buf = a.view(np.float64).reshape(-1) if a.size else np.zeros(1)
        tr = C.byref(trunc.c()) if trunc is not None else None
        h = C.c_void_p()
        L.check(L.lib().tn_mps_from_vector(n if a.size else 0, L.dptr(buf), a.size, tr, PRECISIONS[precision],
                                           int(chi_cap), C.byref(h)), "tn_mps_from_vector")
        return cls(0, _handle=h)

    @classmethod
    def from_parts(cls, gammas, lams, trunc: Trunc | None = None, precision: str = "f64", chi_cap: int = 0):
        """Checkpoint / resume (``tn_mps_import``): a state from its Gamma
        tensors (chi_{k-1}, 2, chi_k) and Lambda vectors in the reference
        layout, as ``export_parts`` returns them."""
        gs = [np.ascontiguousarray(np.asarray(g, dtype=np.complex128)) for g in gammas]
        n = len(gs)
        chi = np.array([1] + [g.shape[2] for g in gs], np.uint32)
        flat = np.concatenate([g.reshape(-1) for g in gs]).view(np.float64) if n else np.zeros(1)
        lam = np.concatenate([np.asarray(x, np.float64).reshape(-1) for x in lams]) if len(lams) else np.zeros(1)
        tr = C.byref(trunc.c()) if trunc is not None else None
        h = C.c_void_p()
        L.check(L.lib().tn_mps_import(n, L.uptr(chi), L.dptr(np.ascontiguousarray(flat)),
                                      L.dptr(np.ascontiguousarray(lam)), tr, PRECISIONS[precision], int(chi_cap),
                                      C.byref(h)), "tn_mps_import")
        return cls(0, _handle=h)

    def export_parts(self):
        """(gammas, lams): every Gamma (chi_{k-1}, 2, chi_k) and Lambda in the
        reference layout (mps.rs:344-353)."""
        return [self.gamma(k) for k in range(self.n)], [self.svals(b) for b in range(self.n - 1)]

    def save(self, path):
        """Write the state, its truncation rule and precision to an npz file."""
        gs, ls = self.export_parts()
        t = self.get_trunc()
        arrays = {f"gamma_{k}": g for k, g in enumerate(gs)}
        arrays.update({f"lambda_{b}": x for b, x in enumerate(ls)})
        np.savez(path, n=self.n, precision=self.precision_name(),
                 trunc=np.array([-1 if t is None else t.mode, 0 if t is None else t.chi_max]),
                 cutoff=0.0 if t is None else t.cutoff, **arrays)

    @classmethod
    def load(cls, path, chi_cap: int = 0):
        """Resume a state written by ``save``."""
        z = np.load(path)
        n = int(z["n"])
        mode, chi_max = (int(x) for x in z["trunc"])
        trunc = None if mode < 0 else Trunc(mode, chi_max, float(z["cutoff"]))
        return cls.from_parts([z[f"gamma_{k}"] for k in range(n)], [z[f"lambda_{b}"] for b in range(n - 1)],
                              trunc, str(z["precision"]), chi_cap)

    def precision_name(self) -> str:
        p = L.i32()
        L.check(self._lib.tn_mps_precision(self._h, C.byref(p)), "tn_mps_precision")
        return {v: k for k, v in PRECISIONS.items()}[int(p.value)]

    def close(self):
        if self._h:
            self._lib.tn_mps_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clone(self) -> "MPS":
        h = C.c_void_p()
        L.check(self._lib.tn_mps_clone(self._h, C.byref(h)), "tn_mps_clone")
        return MPS(0, _handle=h)

    def get_trunc(self):
        t = L.tn_trunc()
        s = L.check(self._lib.tn_mps_get_trunc(self._h, C.byref(t)), "tn_mps_get_trunc")
        return None if s == L.TN_NONE else Trunc(t.mode, t.chi_max, t.cutoff)

    def set_trunc(self, trunc: Trunc | None):
        tr = C.byref(trunc.c()) if trunc is not None else None
        L.check(self._lib.tn_mps_set_trunc(self._h, tr), "tn_mps_set_trunc")

    # ---- unitaries
    def apply_unitary1(self, k: int, op):
        """``apply_unitary1`` (mps.rs:1298-1314)."""
        buf, shape = _as_op(op, 2)
        L.check(self._lib.tn_mps_apply_unitary1(self._h, int(k), L.dptr(buf), shape[0], shape[1]),
                "apply_unitary1")
        return self

    def apply_unitary2(self, k: int, op):
        """``apply_unitary2`` (mps.rs:1332-1387)."""
        buf, shape = _as_op(op, 4)
        L.check(self._lib.tn_mps_apply_unitary2(self._h, int(k), L.dptr(buf), shape[0], shape[1]),
                "apply_unitary2")
        return self

    def apply_gate(self, gate, rng=None):
        """``apply_gate`` / ``apply_gate_rng`` (mps.rs:2044-2069): the gate's
        matrix through ``apply_unitary1`` or ``apply_unitary2``; out-of-range
        qubits are a no-op.  ``rng`` feeds ``Haar2``."""
        k, m = gate.into_matrix(rng)
        if gate.is_q1():
            return self.apply_unitary1(k, m)
        return self.apply_unitary2(k, m)

    def apply_circuit(self, gates, rng=None):
        """``apply_circuit`` / ``apply_circuit_rng`` (mps.rs:2071-2088)."""
        for g in gates:
            self.apply_gate(g, rng)
        return self

    def apply_uni(self, uni, rng=None):
        """``apply_uni`` / ``apply_uni_rng`` (mps.rs:2093-2126): a ``Mat`` must
        be 2x2 or 4x4, otherwise ``TN_ERR_OPERATOR_SHAPE``."""
        if uni.is_gate():
            return self.apply_gate(uni.gate, rng)
        shape = np.shape(uni.matrix)
        if shape == (2, 2):
            return self.apply_unitary1(uni.k, uni.matrix)
        # 4x4 and every other shape: the C ABI answers TN_ERR_OPERATOR_SHAPE for the latter
        return self.apply_unitary2(uni.k, uni.matrix)

    def apply_meas_prob(self, meas, u: float = 0.0):
        """``apply_meas_prob`` (mps.rs:2138-2150): ``Rand`` samples with the
        uniform ``u``, ``Proj`` post-selects; ``None`` when out of range."""
        if meas.is_rand():
            return self.measure_prob(meas.k, u)
        pr = self.measure_postsel_prob(meas.k, meas.outcome)
        return None if pr is None else (meas.outcome, pr)

    def apply_meas(self, meas, u: float = 0.0):
        """``apply_meas`` (mps.rs:2131-2135)."""
        r = self.apply_meas_prob(meas, u)
        return None if r is None else r[0]

    def apply_meas_layer_ops(self, meas, us=None):
        """``apply_meas_prob_layer`` over ``Meas`` values (mps.rs:2206-2252):
        targets are filtered, de-duplicated (first kept) and sorted as there;
        ``us[j]`` is the uniform of the j-th surviving target in ascending
        qubit order (ignored for a ``Proj``)."""
        meas = list(meas)
        ks = [m.k for m in meas]
        posts = [-1 if m.is_rand() else m.outcome for m in meas]
        return self.apply_meas_prob_layer(ks, us if us is not None else np.zeros(len(meas)), posts)

    def apply_bilayer_ops(self, unis, meas, us=None, rng=None):
        """``circuit::apply_bilayer`` (circuit.rs:624-659) over ``Uni`` and
        ``Meas`` sequences: returns (outcomes as ``Meas.proj``, [(k, prob)])."""
        from .gates import Meas
        for u in unis:
            self.apply_uni(u, rng)
        res = self.apply_meas_layer_ops(meas, us)
        return [Meas.proj(k, o) for (k, o, _) in res], [(k, p) for (k, _, p) in res]

    # ---- probabilities / measurement
    def probs(self, k: int):
        """``probs`` (mps.rs:1071-1076)."""
        out = np.zeros(2)
        s = L.check(self._lib.tn_mps_probs(self._h, int(k), L.dptr(out)), "probs")
        return None if s == L.TN_NONE else out

    def prob(self, k: int, p: int):
        out = L.dbl()
        s = L.check(self._lib.tn_mps_prob(self._h, int(k), int(p), C.byref(out)), "prob")
        return None if s == L.TN_NONE else out.value

    def measure_prob(self, k: int, u: float):
        """``measure_prob`` (mps.rs:1479-1489) with the uniform ``u``."""
        oc, pr = L.i32(), L.dbl()
        s = L.check(self._lib.tn_mps_measure_prob(self._h, int(k), float(u), C.byref(oc), C.byref(pr)),
                    "measure_prob")
        return None if s == L.TN_NONE else (int(oc.value), float(pr.value))

    def measure(self, k: int, u: float):
        r = self.measure_prob(k, u)
        return None if r is None else r[0]

    def measure_postsel_prob(self, k: int, p: int):
        """``measure_postsel_prob`` (mps.rs:1501-1510)."""
        pr = L.dbl()
        s = L.check(self._lib.tn_mps_measure_postsel_prob(self._h, int(k), int(p), C.byref(pr)),
                    "measure_postsel_prob")
        return None if s == L.TN_NONE else float(pr.value)

    def measure_postsel(self, k: int, p: int):
        self.measure_postsel_prob(k, p)

    def measure_reset(self, k: int, u: float):
        """``measure_reset`` (mps.rs:2278-2286): measure, then apply the
        reference's ``XMAT`` on outcome 1.  ``XMAT`` is the identity there
        (gate.rs:649-658), so the site is left in the measured state, as in
        the reference."""
        from .gates import make_x
        r = self.measure(k, u)
        if r == 1:
            self.apply_unitary1(k, make_x())
        return r

    def measure_postsel_reset(self, k: int, p: int):
        """``measure_postsel_reset`` (mps.rs:2291-2297), with the same ``XMAT``."""
        from .gates import make_x
        self.measure_postsel(k, p)
        if p != 0:
            self.apply_unitary1(k, make_x())

    def measure_layer(self, ks, us):
        """``measure_layer`` (mps.rs:1519-1548): outcomes of the surviving
        targets (filtered, de-duplicated, ascending); ``us[j]`` is the
        uniform of the j-th of them."""
        return [o for (_, o, _) in self.apply_meas_prob_layer(ks, us)]

    def measure_prob_layer(self, ks, us):
        """``measure_prob_layer`` (mps.rs:1552-1582): [(outcome, prob)]."""
        return [(o, p) for (_, o, p) in self.apply_meas_prob_layer(ks, us)]

    def measure_postsel_prob_layer(self, particles):
        """``measure_postsel_prob_layer`` (mps.rs:1623-1657): ``particles`` =
        [(k, p)]; entries with k >= n or p >= 2 are dropped before the
        de-duplication (first kept), as there; returns the probabilities."""
        keep = [(int(k), int(p)) for (k, p) in particles if 0 <= int(k) < self.n and int(p) in (0, 1)]
        if not keep:
            return []
        res = self.apply_meas_prob_layer([k for k, _ in keep], np.zeros(len(keep)), [p for _, p in keep])
        return [pr for (_, _, pr) in res]

    def measure_postsel_layer(self, particles):
        """``measure_postsel_layer`` (mps.rs:1591-1618)."""
        self.measure_postsel_prob_layer(particles)

    def apply_unitary2_multi(self, k: int, ops):
        """``apply_unitary2_multi`` (mps.rs:1393-1414): the product
        ops[-1] ... ops[0] (4x4 operator constants, multiplied on the host)
        through one ``apply_unitary2``; a no-op for an out-of-range k, and
        ``TN_ERR_OPERATOR_SHAPE`` (nothing applied) if any operator is not 4x4."""
        if self.n == 1 or int(k) >= self.n - 1:
            return self
        acc = np.eye(4, dtype=np.complex128)
        for op in ops:
            op = np.asarray(op, dtype=np.complex128)
            if op.shape != (4, 4):
                raise L.TnError(-5, "apply_unitary2_multi")
            acc = op @ acc
        return self.apply_unitary2(k, acc)

    def apply_op_prob(self, op, u: float = 0.0, rng=None):
        """``apply_op_prob`` (mps.rs:2266-2275): a ``Uni`` is applied (None
        returned), a ``Meas`` measured ((outcome, prob) or None)."""
        from .gates import Meas
        if isinstance(op, Meas):
            return self.apply_meas_prob(op, u)
        self.apply_uni(op, rng)
        return None

    def apply_op(self, op, u: float = 0.0, rng=None):
        """``apply_op`` (mps.rs:2256-2262)."""
        r = self.apply_op_prob(op, u, rng)
        return None if r is None else r[0]

    def apply_meas_prob_layer(self, ks, us=None, posts=None):
        """``apply_meas_prob_layer`` (mps.rs:2206-2252): list of (k, outcome, prob)."""
        ks = np.ascontiguousarray(np.asarray(ks, dtype=np.uint32).reshape(-1))
        nk = ks.size
        usa = None if us is None else np.ascontiguousarray(np.asarray(us, dtype=np.float64).reshape(-1))
        pa = None if posts is None else np.ascontiguousarray(np.asarray(posts, dtype=np.int32).reshape(-1))
        if usa is not None and usa.size < nk:
            usa = np.concatenate([usa, np.zeros(nk - usa.size)])
        ok = np.zeros(max(nk, 1), np.uint32)
        oc = np.zeros(max(nk, 1), np.int32)
        pr = np.zeros(max(nk, 1), np.float64)
        nout = L.u32()
        L.check(self._lib.tn_mps_apply_meas_prob_layer(self._h, L.uptr(ks), nk, L.iptr(pa), L.dptr(usa),
                                                       L.uptr(ok), L.iptr(oc), L.dptr(pr), C.byref(nout)),
                "apply_meas_prob_layer")
        m = nout.value
        return [(int(ok[j]), int(oc[j]), float(pr[j])) for j in range(m)]

    def apply_bilayer(self, gate_ks, gates, meas_ks, us):
        """``circuit::apply_bilayer`` (circuit.rs:624-659), one device launch."""
        gk = np.ascontiguousarray(np.asarray(gate_ks, dtype=np.uint32).reshape(-1))
        g = np.ascontiguousarray(np.asarray(gates, dtype=np.complex128).reshape(-1, 4, 4))
        gbuf = g.view(np.float64).reshape(-1).copy() if g.size else np.zeros(1)
        mk = np.ascontiguousarray(np.asarray(meas_ks, dtype=np.uint32).reshape(-1))
        u = np.ascontiguousarray(np.asarray(us, dtype=np.float64).reshape(-1))
        if u.size < mk.size:
            u = np.concatenate([u, np.zeros(mk.size - u.size)])
        nm = mk.size
        ok = np.zeros(max(nm, 1), np.uint32)
        oc = np.zeros(max(nm, 1), np.int32)
        pr = np.zeros(max(nm, 1), np.float64)
        nout = L.u32()
        L.check(self._lib.tn_mps_apply_bilayer(self._h, L.uptr(gk), L.dptr(gbuf), gk.size, L.uptr(mk), nm,
                                               L.dptr(u if u.size else np.zeros(1)), L.uptr(ok), L.iptr(oc),
                                               L.dptr(pr), C.byref(nout)), "apply_bilayer")
        return [(int(ok[j]), int(oc[j]), float(pr[j])) for j in range(nout.value)]

    # ---- entropies and bonds
    def entropy_vn(self, b: int):
        """``entropy_vn`` (mps.rs:1251-1261)."""
        out = L.dbl()
        s = L.check(self._lib.tn_mps_entropy_vn(self._h, int(b), C.byref(out)), "entropy_vn")
        return None if s == L.TN_NONE else float(out.value)

    def entropy_ry_schmidt(self, a: float, b: int):
        """``entropy_ry_schmidt`` (mps.rs:1268-1282)."""
        out = L.dbl()
        s = L.check(self._lib.tn_mps_entropy_ry_schmidt(self._h, float(a), int(b), C.byref(out)),
                    "entropy_ry_schmidt")
        return None if s == L.TN_NONE else float(out.value)

    def bond_dim(self, b: int):
        out = L.u32()
        s = L.check(self._lib.tn_mps_bond_dim(self._h, int(b), C.byref(out)), "bond_dim")
        return None if s == L.TN_NONE else int(out.value)

    def max_bond_dim(self):
        out = L.u32()
        s = L.check(self._lib.tn_mps_max_bond_dim(self._h, C.byref(out)), "max_bond_dim")
        return None if s == L.TN_NONE else int(out.value)

    def max_bond_dim_idx(self):
        """``max_bond_dim_idx`` (mps.rs:1235-1239): Rust's ``max_by_key`` keeps
        the last of equal maxima."""
        if self.n < 2:
            return None
        dims = [self.bond_dim(b) for b in range(self.n - 1)]
        best = 0
        for b, d in enumerate(dims):
            if d >= dims[best]:
                best = b
        return best

    def svals(self, b: int):
        ln = L.u32()
        s = L.check(self._lib.tn_mps_svals(self._h, int(b), None, 0, C.byref(ln)), "svals")
        if s == L.TN_NONE:
            return None
        out = np.zeros(max(1, ln.value))
        L.check(self._lib.tn_mps_svals(self._h, int(b), L.dptr(out), out.size, C.byref(ln)), "svals")
        return out[: ln.value]

    def gamma(self, k: int):
        """Gamma_k in the reference layout (chi_{k-1}, 2, chi_k), complex128."""
        dims = (L.u32 * 3)()
        s = L.check(self._lib.tn_mps_export_gamma(self._h, int(k), None, 0, dims), "export_gamma")
        if s == L.TN_NONE:
            return None
        shape = (dims[0], dims[1], dims[2])
        out = np.zeros(2 * shape[0] * shape[1] * shape[2])
        L.check(self._lib.tn_mps_export_gamma(self._h, int(k), L.dptr(out), out.size, dims), "export_gamma")
        return out.view(np.complex128).reshape(shape)

    def contract(self):
        """``contract`` (mps.rs:794-798): dense state vector (n <= 24)."""
        out = np.zeros(2 * (1 << self.n))
        L.check(self._lib.tn_mps_contract(self._h, L.dptr(out), out.size), "contract")
        return out.view(np.complex128)

    def stats(self, reset: bool = False):
        """Device work counters: theta flops, SVD flops, bond ops, Jacobi
        sweeps, measurements, algorithmic bytes."""
        out = np.zeros(16)
        L.check(self._lib.tn_mps_stats(self._h, L.dptr(out), int(reset)), "stats")
        return dict(flop_theta=out[0], flop_svd=out[1], bond_ops=out[2], sweeps=out[3], meas=out[4], bytes=out[5],
                    cyc_theta=out[6], cyc_gram=out[7], cyc_rot=out[8], cyc_update=out[9], cyc_final=out[10],
                    block_steps=out[11], lq_ops=out[12], nonconv=out[13], nonconv_c_lq=out[14],
                    nonconv_c_direct=out[15])

    def device_status(self) -> int:
        st = L.i32()
        L.check(self._lib.tn_mps_device_status(self._h, C.byref(st)), "device_status")
        return int(st.value)
