"""Batch of independent trajectories over ``tn_batch_*`` (one persistent
launch per brickwork layer for every listed trajectory)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .mps import PRECISIONS, Trunc


class Batch:
    def __init__(self, ns, truncs=None, precision: str = "mixed", chi_caps=None):
        self._lib = L.lib()
        ns = np.ascontiguousarray(np.asarray(ns, dtype=np.uint32))
        self.ntraj = int(ns.size)
        self.ns = ns.copy()
        tarr = None
        if truncs is not None:
            tarr = (L.tn_trunc * self.ntraj)(*[t.c() for t in truncs])
        caps = None if chi_caps is None else np.ascontiguousarray(np.asarray(chi_caps, dtype=np.uint32))
        self._h = C.c_void_p()
        L.check(self._lib.tn_batch_create(self.ntraj, L.uptr(ns), tarr, PRECISIONS[precision], L.uptr(caps),
                                          C.byref(self._h)), "tn_batch_create")

    def close(self):
        if self._h:
            self._lib.tn_batch_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self, t: int, n: int, trunc: Trunc | None):
        tr = C.byref(trunc.c()) if trunc is not None else None
        L.check(self._lib.tn_batch_reset(self._h, int(t), int(n), tr), "tn_batch_reset")
        self.ns[t] = n

    def import_state(self, t: int, gammas, lams, trunc: Trunc | None):
        """Slot t := the state given by its Gamma / Lambda parts in the
        reference layout (``tn_batch_import``), e.g. ``MPS.export_parts()``."""
        gs = [np.ascontiguousarray(np.asarray(g, dtype=np.complex128)) for g in gammas]
        n = len(gs)
        chi = np.array([1] + [g.shape[2] for g in gs], np.uint32)
        flat = np.ascontiguousarray(np.concatenate([g.reshape(-1) for g in gs]).view(np.float64))
        lam = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64).reshape(-1) for x in lams])
                                   if len(lams) else np.zeros(1))
        tr = C.byref(trunc.c()) if trunc is not None else None
        L.check(self._lib.tn_batch_import(self._h, int(t), n, L.uptr(chi), L.dptr(flat), L.dptr(lam), tr),
                "tn_batch_import")
        self.ns[t] = n

    def gamma(self, t: int, k: int):
        dims = (L.u32 * 3)()
        s = L.check(self._lib.tn_batch_export_gamma(self._h, int(t), int(k), None, 0, dims), "export_gamma")
        if s == L.TN_NONE:
            return None
        shape = (dims[0], dims[1], dims[2])
        out = np.zeros(2 * shape[0] * shape[1] * shape[2])
        L.check(self._lib.tn_batch_export_gamma(self._h, int(t), int(k), L.dptr(out), out.size, dims),
                "export_gamma")
        return out.view(np.complex128).reshape(shape)

    def export_parts(self, t: int):
        n = int(self.ns[t])
        return [self.gamma(t, k) for k in range(n)], [self.svals(t, b) for b in range(n - 1)]

    @staticmethod
    def pack(trajs, layers):
        """layers[i] = (gate_ks, gates[ng,4,4] complex, meas_ks sorted, us)."""
        gate_off = [0]
        meas_off = [0]
        gks, gs, mks, uss = [], [], [], []
        for (gk, g, mk, us) in layers:
            gk = np.asarray(gk, dtype=np.uint32).reshape(-1)
            gks.append(gk)
            gs.append(np.asarray(g, dtype=np.complex128).reshape(-1, 4, 4))
            mks.append(np.asarray(mk, dtype=np.uint32).reshape(-1))
            uss.append(np.asarray(us, dtype=np.float64).reshape(-1))
            gate_off.append(gate_off[-1] + gk.size)
            meas_off.append(meas_off[-1] + mks[-1].size)
        cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs).astype(dt)) if xs else np.zeros(0, dt)
        return dict(
            trajs=np.ascontiguousarray(np.asarray(trajs, dtype=np.uint32)),
            gate_off=np.asarray(gate_off, np.uint32), gate_ks=cat(gks, np.uint32),
            gates=np.ascontiguousarray(np.concatenate(gs).view(np.float64).reshape(-1)) if gs else np.zeros(0),
            meas_off=np.asarray(meas_off, np.uint32), meas_ks=cat(mks, np.uint32), us=cat(uss, np.float64))

    def step_packed(self, pk, posts=None):
        """posts (optional, parallel to pk["meas_ks"]): 0 / 1 post-selects that
        outcome (Meas::Proj), -1 samples with the uniform (Meas::Rand)."""
        nt = pk["trajs"].size
        nm = int(pk["meas_off"][-1])
        oc = np.zeros(max(nm, 1), np.int32)
        pr = np.zeros(max(nm, 1), np.float64)
        ent = np.zeros(max(nt, 1), np.float64)
        z = np.zeros(1)
        zu = np.zeros(1, np.uint32)
        args = [self._h, L.uptr(pk["trajs"]), nt, L.uptr(pk["gate_off"]),
                L.uptr(pk["gate_ks"] if pk["gate_ks"].size else zu),
                L.dptr(pk["gates"] if pk["gates"].size else z), L.uptr(pk["meas_off"]),
                L.uptr(pk["meas_ks"] if pk["meas_ks"].size else zu), L.dptr(pk["us"] if pk["us"].size else z)]
        if posts is None:
            L.check(self._lib.tn_batch_step(*args, L.iptr(oc), L.dptr(pr), L.dptr(ent)), "tn_batch_step")
        else:
            ps = np.ascontiguousarray(np.asarray(posts, dtype=np.int32).reshape(-1))
            assert ps.size == nm
            zi = np.full(1, -1, np.int32)
            L.check(self._lib.tn_batch_step_post(*args, L.iptr(ps if ps.size else zi), L.iptr(oc), L.dptr(pr),
                                                 L.dptr(ent)), "tn_batch_step_post")
        return oc[:nm], pr[:nm], ent[:nt]

    def step(self, trajs, layers, posts=None):
        """Advance each listed trajectory by its layer; returns per-trajectory
        lists of (k, outcome, prob) and the half-chain entropies.  posts[i]
        (optional) gives trajectory i's post-selected outcomes, parallel to its
        sorted measurement sites (-1 = sample)."""
        pk = self.pack(trajs, layers)
        flat = None if posts is None else np.concatenate([np.asarray(x, np.int32).reshape(-1) for x in posts]
                                                         or [np.zeros(0, np.int32)])
        oc, pr, ent = self.step_packed(pk, flat)
        recs = []
        mo = pk["meas_off"]
        for i in range(len(trajs)):
            recs.append([(int(pk["meas_ks"][j]), int(oc[j]), float(pr[j])) for j in range(mo[i], mo[i + 1])])
        return recs, ent

    def bond_dims(self, t: int):
        n = int(self.ns[t])
        out = np.zeros(max(1, n - 1), np.uint32)
        s = L.check(self._lib.tn_batch_bond_dims(self._h, int(t), L.uptr(out), out.size), "bond_dims")
        return None if s == L.TN_NONE else out[: n - 1]

    def svals(self, t: int, b: int):
        ln = L.u32()
        s = L.check(self._lib.tn_batch_svals(self._h, int(t), int(b), None, 0, C.byref(ln)), "svals")
        if s == L.TN_NONE:
            return None
        out = np.zeros(max(1, ln.value))
        L.check(self._lib.tn_batch_svals(self._h, int(t), int(b), L.dptr(out), out.size, C.byref(ln)), "svals")
        return out[: ln.value]

    def device_status(self) -> int:
        st = L.i32()
        L.check(self._lib.tn_batch_device_status(self._h, C.byref(st)), "device_status")
        return int(st.value)

    def stats(self, reset: bool = False):
        out = np.zeros(16)
        L.check(self._lib.tn_batch_stats(self._h, L.dptr(out), int(reset)), "stats")
        return dict(flop_theta=out[0], flop_svd=out[1], bond_ops=out[2], sweeps=out[3], meas=out[4], bytes=out[5],
                    cyc_theta=out[6], cyc_gram=out[7], cyc_rot=out[8], cyc_update=out[9], cyc_final=out[10],
                    block_steps=out[11], lq_ops=out[12], nonconv=out[13], nonconv_c_lq=out[14],
                    nonconv_c_direct=out[15])

    def step_ptrs(self, nt, trajs, order, gate_off, gate_ks, gates, meas_off, meas_ks, us, outcomes, probs, entropy):
        """Layer step from device pointers (ints: int32, reals: float64)."""
        L.check(self._lib.tn_batch_step_ptrs(self._h, int(nt), trajs, order, gate_off, gate_ks, gates, meas_off,
                                             meas_ks, us, outcomes, probs, entropy), "tn_batch_step_ptrs")

    _INPUT_NAMES = ("trajs", "gate_off", "gate_ks", "gates", "meas_off", "meas_ks", "us", "outcomes", "probs",
                    "entropy")

    def device_inputs(self, max_gates: int, max_meas: int):
        """Device buffers of the graph-captured step (tn_batch_device_inputs):
        name -> device pointer (int32 indices, float64 gates/uniforms)."""
        ptrs = [C.c_void_p() for _ in self._INPUT_NAMES]
        L.check(self._lib.tn_batch_device_inputs(self._h, int(max_gates), int(max_meas),
                                                 *[C.byref(p) for p in ptrs]), "tn_batch_device_inputs")
        return {k: int(p.value) for k, p in zip(self._INPUT_NAMES, ptrs)}

    def step_device(self, nt: int):
        """Replay the captured layer launch for the first nt listed trajectories
        (stream-ordered on the batch stream, no synchronisation)."""
        L.check(self._lib.tn_batch_step_device(self._h, int(nt)), "tn_batch_step_device")

    def slot_bytes(self, t: int) -> int:
        b = L.u64()
        L.check(self._lib.tn_batch_slot_bytes(self._h, int(t), C.byref(b)), "slot_bytes")
        return int(b.value)

    def stream(self) -> int:
        s = C.c_void_p()
        L.check(self._lib.tn_batch_stream(self._h, C.byref(s)), "stream")
        return int(s.value or 0)

    def set_tuning(self, scheme: int = 0, max_sweeps: int = 40):
        L.check(self._lib.tn_batch_set_tuning(self._h, int(scheme), int(max_sweeps)), "set_tuning")

    def set_schedule(self, schedule: int = 1):
        """1: one launch per layer (sweeps pushed as their gates finish); 0: two launches."""
        L.check(self._lib.tn_batch_set_schedule(self._h, int(schedule)), "set_schedule")

    def set_theta_path(self, simt: bool = False):
        """Mixed precision: SIMT FP32 theta contraction (True) or tensor cores (False, default)."""
        L.check(self._lib.tn_batch_set_theta_path(self._h, int(bool(simt))), "set_theta_path")

    def autotune(self, trial_steps: int = 1):
        """Tune schedule / Jacobi scheme / theta path over the next 4 * trial_steps steps."""
        L.check(self._lib.tn_batch_autotune(self._h, int(trial_steps)), "autotune")

    def tuning(self):
        cfg = (L.i32 * 4)()
        sc = np.zeros(4)
        L.check(self._lib.tn_batch_tuning(self._h, cfg, L.dptr(sc)), "tuning")
        return dict(schedule=cfg[0], scheme=cfg[1], theta_simt=cfg[2], tuning=bool(cfg[3]), scores=list(sc))

    def last_launch_ms(self):
        """(gate launch ms, sweep launch ms) of the last non-graph step; with
        the one-launch schedule the first is the whole launch and the second 0."""
        g, w = C.c_float(), C.c_float()
        s = L.check(self._lib.tn_batch_last_launch_ms(self._h, C.byref(g), C.byref(w)), "last_launch_ms")
        return None if s == L.TN_NONE else (g.value, w.value)

    def set_queue_wait(self, wait_ns: int = 0, phantom_sweeps: int = 0):
        """Limit of a CTA's wait for a pushed sweep item (0: 120 s) and sweep
        slots that no item fills (to make that wait run out in a test)."""
        L.check(self._lib.tn_batch_set_queue_wait(self._h, int(wait_ns), int(phantom_sweeps)), "set_queue_wait")

    def last_step_device_ms(self):
        """Device time of the last host-input step from the end of its input
        copy to the start of its output copy (every kernel of the layer)."""
        ms = C.c_float()
        s = L.check(self._lib.tn_batch_last_step_device_ms(self._h, C.byref(ms)), "last_step_device_ms")
        return None if s == L.TN_NONE else ms.value

    def synchronize(self):
        L.check(self._lib.tn_batch_synchronize(self._h), "synchronize")
