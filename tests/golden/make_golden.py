"""Writes tests/golden/trajectories.npz: seeded brickwork trajectories (inputs
from the counter-based generator) and the FP64 oracle's results on them --
per-layer half-chain entropies, measurement records and the final Schmidt
values of every bond.  The GPU parity tests compare against these arrays, so
the oracle does not have to run at test time.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402
from oracle import mps_ref as R  # noqa: E402

# (name, n, chi_max, cutoff, p, depth, seed, traj)
CASES = [
    ("n8_chi16_p20", 8, 16, 1e-12, 0.20, 10, 11, 0),
    ("n10_chi8_p10", 10, 8, 1e-12, 0.10, 12, 11, 1),
    ("n12_chi32_p05", 12, 32, 1e-10, 0.05, 10, 12, 2),
    ("n6_chi4_p30", 6, 4, 1e-12, 0.30, 10, 13, 3),
    ("n9_chi64_p15", 9, 64, 1e-10, 0.15, 8, 14, 4),
]


def main():
    tn = ge.load_package()
    out = {}
    for name, n, chi, cutoff, p, depth, seed, traj in CASES:
        layers = tn.gen_trajectory(seed, traj, n, depth, p)
        m = R.MPS(n, R.Trunc.both(chi, cutoff))
        ents, rk, ro, rp, roff = [], [], [], [], [0]
        for (gk, g, mk, us) in layers:
            rec = R.apply_bilayer(m, gk, g, mk, us)
            ents.append(m.entropy_vn(n // 2 - 1))
            for (k, o, pr) in rec:
                rk.append(k)
                ro.append(o)
                rp.append(pr)
            roff.append(len(rk))
        gko = np.cumsum([0] + [len(L[0]) for L in layers])
        mko = np.cumsum([0] + [len(L[2]) for L in layers])
        sv = [np.asarray(s, dtype=np.float64) for s in m.svals]
        svo = np.cumsum([0] + [len(s) for s in sv])
        out.update({
            f"{name}/spec": np.array([n, chi, depth, seed, traj], dtype=np.int64),
            f"{name}/cutoff_p": np.array([cutoff, p]),
            f"{name}/gate_ks": np.concatenate([L[0] for L in layers]).astype(np.int32),
            f"{name}/gate_off": gko.astype(np.int32),
            f"{name}/gates": np.concatenate([L[1].reshape(-1, 4, 4) for L in layers]).astype(np.complex128),
            f"{name}/meas_ks": np.concatenate([L[2] for L in layers]).astype(np.int32),
            f"{name}/meas_off": mko.astype(np.int32),
            f"{name}/us": np.concatenate([L[3] for L in layers]).astype(np.float64),
            f"{name}/entropy": np.asarray(ents, dtype=np.float64),
            f"{name}/rec_k": np.asarray(rk, dtype=np.int32),
            f"{name}/rec_outcome": np.asarray(ro, dtype=np.int32),
            f"{name}/rec_prob": np.asarray(rp, dtype=np.float64),
            f"{name}/rec_off": np.asarray(roff, dtype=np.int32),
            f"{name}/svals": np.concatenate(sv),
            f"{name}/svals_off": svo.astype(np.int32),
        })
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "trajectories.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
