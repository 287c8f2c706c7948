"""Circuit files in the reference's npz layout (workspace/lib/haar.rs:54-101,
`save_unis` / `load_unis`): arrays `depth` (uint32, layer of each gate),
`targs` (uint32, left qubit of each gate) and `mats` (complex128, one 4x4
matrix per gate), gates of a layer contiguous.  Loading groups consecutive
entries with equal depth into one layer, as `load_unis` does (a depth with no
gate yields no layer).  The layers feed `MPS.apply_bilayer`, `Batch.step` or
`tn_batch_step` directly."""
from __future__ import annotations

import numpy as np


def save_unis(path, layers):
    """layers[t] = (gate_ks, gates[ng, 4, 4]) -> npz with depth / targs / mats."""
    depth, targs, mats = [], [], []
    for t, (gk, g) in enumerate(layers):
        g = np.asarray(g, dtype=np.complex128).reshape(-1, 4, 4)
        for k, m in zip(np.asarray(gk).reshape(-1), g):
            depth.append(t)
            targs.append(int(k))
            mats.append(m)
    np.savez(path, depth=np.asarray(depth, np.uint32), targs=np.asarray(targs, np.uint32),
             mats=np.asarray(mats, np.complex128).reshape(-1, 4, 4))


def load_unis(path):
    """npz (depth, targs, mats) -> [(gate_ks uint32[ng], gates complex128[ng, 4, 4]), ...]."""
    z = np.load(path)
    depth = np.asarray(z["depth"]).astype(np.int64).reshape(-1)
    targs = np.asarray(z["targs"]).astype(np.uint32).reshape(-1)
    mats = np.asarray(z["mats"]).astype(np.complex128).reshape(-1, 4, 4)
    if not (len(depth) == len(targs) == len(mats)):
        raise ValueError("depth, targs and mats must have one entry per gate")
    layers = []
    i = 0
    while i < len(depth):
        j = i
        while j < len(depth) and depth[j] == depth[i]:
            j += 1
        layers.append((targs[i:j].copy(), mats[i:j].copy()))
        i = j
    return layers
