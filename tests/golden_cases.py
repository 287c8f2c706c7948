"""Loader of the committed golden trajectories (tests/golden/trajectories.npz,
written by tests/golden/make_golden.py from the FP64 oracle)."""
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "trajectories.npz")


def load():
    z = np.load(PATH)
    names = sorted({k.split("/")[0] for k in z.files})
    cases = []
    for nm in names:
        g = lambda key: z[f"{nm}/{key}"]
        n, chi, depth, seed, traj = (int(x) for x in g("spec"))
        cutoff, p = (float(x) for x in g("cutoff_p"))
        go, mo, ro, so = g("gate_off"), g("meas_off"), g("rec_off"), g("svals_off")
        layers = [(g("gate_ks")[go[t]:go[t + 1]].astype(np.uint32), g("gates")[go[t]:go[t + 1]],
                   g("meas_ks")[mo[t]:mo[t + 1]].astype(np.uint32), g("us")[mo[t]:mo[t + 1]]) for t in range(depth)]
        recs = [[(int(g("rec_k")[j]), int(g("rec_outcome")[j]), float(g("rec_prob")[j])) for j in range(ro[t], ro[t + 1])]
                for t in range(depth)]
        svals = [g("svals")[so[b]:so[b + 1]] for b in range(n - 1)]
        cases.append(dict(name=nm, n=n, chi=chi, depth=depth, seed=seed, traj=traj, cutoff=cutoff, p=p,
                          layers=layers, entropy=g("entropy"), recs=recs, svals=svals))
    return cases
