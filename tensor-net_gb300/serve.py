"""Continuous-batching trajectory server over ``tn_server_*`` and a Poisson
load generator (the serving workload: arrivals at a mean rate, n log-uniform,
chi_max log-uniform over powers of two, p uniform, depth uniform in
[2n, 4n])."""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import _lib as L
from .mps import PRECISIONS, Trunc


class Server:
    """Requests with bond capacity <= light_chi run in class 0 on light_ctas
    CTAs, the rest in class 1 on the remaining SMs; the classes step
    independently (0 = defaults: 64 and a fifth of the SMs)."""

    def __init__(self, hbm_bytes: int, max_slots: int = 1024, precision: str = "mixed", max_chi: int = 512,
                 max_n: int = 128, light_chi: int = 0, light_ctas: int = 0):
        self._lib = L.lib()
        self._h = C.c_void_p()
        L.check(self._lib.tn_server_create_classes(int(hbm_bytes), int(max_slots), PRECISIONS[precision],
                                                   int(max_chi), int(max_n), int(light_chi), int(light_ctas),
                                                   C.byref(self._h)), "tn_server_create_classes")

    def close(self):
        if self._h:
            self._lib.tn_server_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def now(self) -> float:
        t = L.dbl()
        L.check(self._lib.tn_server_now(self._h, C.byref(t)), "tn_server_now")
        return t.value

    def submit(self, n, trunc: Trunc, p, depth, seed, traj, arrival=-1.0) -> int:
        r = L.tn_request(int(n), trunc.c(), float(p), int(depth), int(seed), int(traj))
        i = L.u64()
        L.check(self._lib.tn_server_submit(self._h, C.byref(r), float(arrival), C.byref(i)), "tn_server_submit")
        return int(i.value)

    def tick(self):
        a, d = L.u32(), L.u32()
        L.check(self._lib.tn_server_tick(self._h, C.byref(a), C.byref(d)), "tn_server_tick")
        return int(a.value), int(d.value)

    def poll(self, cap: int = 4096, history: bool = False):
        """Retired requests; with ``history`` each result also carries
        ``entropies``, the half-chain entropy after every layer
        (``tn_server_history``)."""
        buf = (L.tn_result * cap)()
        n = L.u32()
        L.check(self._lib.tn_server_poll(self._h, buf, cap, C.byref(n)), "tn_server_poll")
        out = [dict(id=r.id, layers=r.layers, final_entropy=r.final_entropy, latency_s=r.latency_s,
                    queue_s=r.queue_s, status=r.status) for r in buf[: n.value]]
        if history:
            for d in out:
                d["entropies"] = self.history(d["id"])
        return out

    def history(self, req_id: int):
        ln = L.u32()
        s = L.check(self._lib.tn_server_history(self._h, int(req_id), None, 0, C.byref(ln)), "tn_server_history")
        if s == L.TN_NONE:
            return None
        buf = np.zeros(max(1, ln.value))
        L.check(self._lib.tn_server_history(self._h, int(req_id), L.dptr(buf), buf.size, C.byref(ln)),
                "tn_server_history")
        return buf[: ln.value].copy()

    def cancel(self, req_id: int) -> bool:
        """Cancel a queued or resident request (``tn_server_cancel``); its
        result (status ``TN_CANCELLED``) appears in ``poll``.  False when the
        id is unknown or already finished."""
        s = L.check(self._lib.tn_server_cancel(self._h, int(req_id)), "tn_server_cancel")
        return s == L.TN_OK

    def stats(self):
        out = np.zeros(8)
        L.check(self._lib.tn_server_stats(self._h, L.dptr(out)), "tn_server_stats")
        return dict(layers=out[0], busy_s=out[1], ticks=out[2], arena_used=out[3], pending=out[4], active=out[5],
                    admitted=out[6], completed=out[7])

    def set_policy(self, policy: str = "fcfs", max_active=(0, 0)):
        """Admission order within a class ("fcfs" or "least-work") and the
        cap on resident requests per class (0 = every slot)."""
        L.check(self._lib.tn_server_set_policy(self._h, {"fcfs": 0, "least-work": 1}[policy], int(max_active[0]),
                                               int(max_active[1])), "tn_server_set_policy")

    def class_stats(self, cls: int):
        out = np.zeros(6)
        L.check(self._lib.tn_server_class_stats(self._h, int(cls), L.dptr(out)), "tn_server_class_stats")
        return dict(cap_max=int(out[0]), ctas=int(out[1]), layers=out[2], launches=out[3], pending=int(out[4]),
                    active=int(out[5]))


def poisson_requests(rate, duration, seed, n_range=(16, 128), chis=(64, 128, 256, 512), p_range=(0.02, 0.3),
                     cutoff=1e-10):
    """Arrival times and request parameters of the serving workload."""
    rng = np.random.default_rng(seed)
    t, out, i = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        chi = int(chis[rng.integers(len(chis))])
        p = float(rng.uniform(*p_range))
        depth = int(rng.integers(2 * n, 4 * n + 1))
        out.append(dict(t=t, n=n, chi=chi, p=p, depth=depth, traj=i, cutoff=cutoff))
        i += 1
    return out


def run_poisson(server: Server, reqs, duration: float, seed: int, drain: bool = False):
    """Drive the server in real time: submit every request whose arrival time
    has passed, tick, collect completions; stop at `duration` seconds (or
    when everything completed, with drain=True)."""
    t0 = server.now()
    k = 0
    done = []
    while True:
        now = server.now() - t0
        while k < len(reqs) and reqs[k]["t"] <= now:
            r = reqs[k]
            server.submit(r["n"], Trunc.both(r["chi"], r["cutoff"]), r["p"], r["depth"], seed, r["traj"],
                          arrival=t0 + r["t"])
            k += 1
        a, _ = server.tick()
        done += server.poll()
        if now >= duration and not drain:
            break
        if drain and k == len(reqs) and a == 0:
            break
        if a == 0 and k < len(reqs):
            wait = reqs[k]["t"] - (server.now() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.05))
    return done, k
