"""Seeded brickwork inputs for the CPU side of the benchmarks, in plain Python.

TEST INFRASTRUCTURE ONLY (like ``mps_ref``): used by ``tests/`` and by the CPU
legs of ``bench.py`` (``cpu_baseline`` and ``--impl reference``) so that the
reference arm produces the GPU arm's inputs without loading the product
library.

A step-by-step restatement of the library's input generator
(``tensor-net_gb300/csrc/tn_gen.cpp``), which ``tests/test_gen_ref.py`` holds
bit for bit to ``tn_gen_layer``:

* SplitMix64 mixing (Steele, Lea and Flood 2014) of (seed, trajectory, layer,
  site, purpose, index) into 64-bit keys; uniforms from the top 53 bits;
* Box-Muller normals (Box and Muller 1958) for the complex Ginibre 4x4 sample
  of ``gate::haar`` (tensor-net/lib/gate.rs:888-909), filled row-major with
  (re, im) pairs;
* QR by modified Gram-Schmidt with one re-orthogonalisation pass, which gives
  the unique Q with a positive real R diagonal, i.e. Q divided column-wise by
  r_jj / |r_jj| as gate.rs:902-907 does;
* the TileQ2 gate positions of layer t (offset t odd, circuit.rs:523-531,
  workspace/lib/haar.rs:285) and ``uniform_meas`` (circuit.rs:580-584): site k
  measured iff its location uniform is below p, with one outcome uniform each.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = (1 << 64) - 1
P_GATE, P_LOC, P_OUT = 1, 2, 3


def mix64(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & _M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return z ^ (z >> 31)


def key(seed: int, traj: int, layer: int, site: int, purpose: int, idx: int) -> int:
    h = mix64((seed ^ 0x5851F42D4C957F2D) & _M64)
    h = mix64(h ^ (traj & _M64))
    h = mix64(h ^ (((layer & 0xFFFFFFFF) << 32) | (site & 0xFFFFFFFF)))
    h = mix64(h ^ (((purpose << 56) | idx) & _M64))
    return h


def unif(k: int) -> float:
    """Uniform in [0, 1) with 53 random bits."""
    return float(k >> 11) * (1.0 / 9007199254740992.0)


def normal_pair(k: int):
    u1 = 1.0 - unif(mix64(k ^ 0x1))  # (0, 1]
    u2 = unif(mix64(k ^ 0x2))
    r = math.sqrt(-2.0 * math.log(u1))
    th = 6.283185307179586 * u2
    return r * math.cos(th), r * math.sin(th)


def _cmul(a, b):
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def haar_u4(z):
    """Q of the Ginibre sample z (4x4 complex, row-major) with a positive real
    R diagonal, by the operation order of the C++ generator."""
    a = [[(float(z[r][c].real), float(z[r][c].imag)) for c in range(4)] for r in range(4)]
    q = [[(0.0, 0.0)] * 4 for _ in range(4)]
    for j in range(4):
        v = [a[r][j] for r in range(4)]
        for _ in range(2):
            for i in range(j):
                dr, di = 0.0, 0.0  # q_i^H v
                for r in range(4):
                    t = _cmul((q[r][i][0], -q[r][i][1]), v[r])
                    dr += t[0]
                    di += t[1]
                for r in range(4):
                    t = _cmul((dr, di), q[r][i])
                    v[r] = (v[r][0] - t[0], v[r][1] - t[1])
        nrm = 0.0
        for r in range(4):
            nrm += v[r][0] * v[r][0] + v[r][1] * v[r][1]
        nrm = math.sqrt(nrm)
        if not nrm > 0.0:
            raise ValueError("singular Ginibre sample")
        for r in range(4):
            q[r][j] = (v[r][0] / nrm, v[r][1] / nrm)
    return np.array([[complex(*q[r][c]) for c in range(4)] for r in range(4)], dtype=np.complex128)


def ginibre(seed: int, traj: int, layer: int, site: int):
    z = np.zeros((4, 4), dtype=np.complex128)
    for e in range(16):
        re, im = normal_pair(key(seed, traj, layer, site, P_GATE, e))
        z[e // 4, e % 4] = complex(re, im)
    return z


def gen_layer(seed: int, traj: int, layer: int, n: int, p: float):
    """(gate_ks, gates[ng,4,4], meas_ks, us) of one brickwork layer."""
    if n == 0:
        raise ValueError("EmptySystem")
    gks, gates = [], []
    for k in range(layer & 1, n - 1, 2):
        gks.append(k)
        gates.append(haar_u4(ginibre(seed, traj, layer, k)))
    mks, us = [], []
    for k in range(n):
        if unif(key(seed, traj, layer, k, P_LOC, 0)) < p:
            mks.append(k)
            us.append(unif(key(seed, traj, layer, k, P_OUT, 0)))
    g = np.array(gates, dtype=np.complex128).reshape(len(gates), 4, 4)
    return np.array(gks, np.uint32), g, np.array(mks, np.uint32), np.array(us, np.float64)


def gen_trajectory(seed: int, traj: int, n: int, depth: int, p: float):
    return [gen_layer(seed, traj, t, n, p) for t in range(depth)]
