"""Seeded synthetic brickwork inputs (``tn_gen_layer`` / ``tn_haar_u4``).

Haar-random U(4) gates (gate::haar, tensor-net/lib/gate.rs:888-909) at the
TileQ2 positions of layer t (circuit.rs:523-563, offset = t odd), and the
Bernoulli(p) measurement layer of uniform_meas (circuit.rs:580-584) with one
outcome uniform per measured site.  Every value is a function of
(seed, traj, layer, site), so CPU and GPU consume identical arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def haar_u4(z):
    """QR-based Haar unitary from a 4x4 complex Ginibre sample."""
    zz = np.ascontiguousarray(np.asarray(z, dtype=np.complex128).reshape(4, 4)).view(np.float64).reshape(-1)
    out = np.zeros(32)
    L.check(L.lib().tn_haar_u4(L.dptr(zz), L.dptr(out)), "tn_haar_u4")
    return out.view(np.complex128).reshape(4, 4)


def ginibre(seed: int, traj: int, layer: int, site: int):
    out = np.zeros(32)
    L.check(L.lib().tn_gen_ginibre(int(seed), int(traj), int(layer), int(site), L.dptr(out)), "tn_gen_ginibre")
    return out.view(np.complex128).reshape(4, 4)


def gen_layer(seed: int, traj: int, layer: int, n: int, p: float):
    """(gate_ks, gates[ng,4,4], meas_ks, us) of one brickwork layer."""
    gk = np.zeros(max(1, n), np.uint32)
    g = np.zeros(32 * max(1, n // 2 + 1))
    mk = np.zeros(max(1, n), np.uint32)
    us = np.zeros(max(1, n))
    ng, nm = L.u32(), L.u32()
    L.check(L.lib().tn_gen_layer(int(seed), int(traj), int(layer), int(n), float(p), L.uptr(gk), L.dptr(g),
                                 C.byref(ng), L.uptr(mk), L.dptr(us), C.byref(nm)), "tn_gen_layer")
    a, b = ng.value, nm.value
    return gk[:a].copy(), g[: 32 * a].view(np.complex128).reshape(a, 4, 4).copy(), mk[:b].copy(), us[:b].copy()


def gen_trajectory(seed: int, traj: int, n: int, depth: int, p: float):
    return [gen_layer(seed, traj, t, n, p) for t in range(depth)]
