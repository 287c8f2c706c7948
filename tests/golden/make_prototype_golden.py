"""Writes tests/golden/prototype.npz: outputs of the reference's own Python
prototypes (prototyping/haar-unitary.py, prototyping/schmidt_mps.py in the
reference tree), run here on seeded inputs, for the CPU tests that pin the
oracle to code the reference ships.

* haar: ``random_haar(2)`` from haar-unitary.py with numpy's global generator
  seeded; the 32 normals it draws are recorded (in draw order: re, im of
  element 0, 1, ...), so a test can hand the same Ginibre matrix to the
  oracle's Haar recipe.
* schmidt: ``canonicalize(n, psi)`` from schmidt_mps.py on seeded complex
  Gaussian states, n = 2..8: the Schmidt values of every bond, and
  ``contract`` of the result (the prototype's own state vector).
* gate2: n = 2 only, ``apply_2q(canonicalize(2, psi), 0, U)``: the Schmidt
  values after a Haar gate.  (The prototype's ``apply_2q`` leaves out the
  outer Lambdas of theta, which is exact only for two qubits.)
* gate1: ``apply_1q`` of a one-qubit Haar gate on one site (exact for any n):
  the contracted state.
* entropy: ``entropy_log`` of the reduced density matrix (``trace_qubit``)
  from prototyping/entropy.py, for every bond of the n = 4, 6, 8 states.
* proj: ``project(mps, k, p)`` where the prototype's contraction spans the
  whole chain (n = 2; the middle site of n = 3): Schmidt values and state
  (the middle-site branch's state does not contract back to the projected
  vector; its Schmidt values are right).

haar-unitary.py plots at import time and imports a plotting package that is
not installed, so only its ``random_haar`` definition is compiled (taken from
the file's syntax tree); schmidt_mps.py is imported as a module.

    python tests/golden/make_prototype_golden.py
"""
import ast
import importlib.util
import os
import pathlib

import numpy as np

PROTO = pathlib.Path(os.environ.get("TN_REFERENCE_ROOT", "/root/reference")) / "prototyping"
OUT = pathlib.Path(__file__).resolve().parent / "prototype.npz"


def _random_haar():
    src = (PROTO / "haar-unitary.py").read_text()
    tree = ast.parse(src)
    fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "random_haar"]
    mod = ast.Module(body=fn, type_ignores=[])
    ns = {"np": np}
    exec(compile(mod, str(PROTO / "haar-unitary.py"), "exec"), ns)
    return ns["random_haar"]


def _defs(fname, names, ns):
    """Compile only the named top-level definitions of a prototype script
    (the scripts print or plot at import time)."""
    src = (PROTO / fname).read_text()
    body = [n for n in ast.parse(src).body if isinstance(n, ast.FunctionDef) and n.name in names]
    exec(compile(ast.Module(body=body, type_ignores=[]), str(PROTO / fname), "exec"), ns)
    return ns


def _schmidt_mps():
    spec = importlib.util.spec_from_file_location("schmidt_mps", PROTO / "schmidt_mps.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def main():
    random_haar = _random_haar()
    sm = _schmidt_mps()
    out = {}

    # haar: the prototype's recipe on recorded normals
    draws = []
    real_normal = np.random.normal

    def recording_normal(*args, **kw):
        x = real_normal(*args, **kw)
        draws.append(float(x))
        return x

    hs, zs = [], []
    for i in range(8):
        np.random.seed(9100 + i)
        draws.clear()
        np.random.normal = recording_normal
        try:
            u = random_haar(2)
        finally:
            np.random.normal = real_normal
        d = np.asarray(draws).reshape(16, 2)
        zs.append((d[:, 0] + 1j * d[:, 1]).reshape(4, 4))
        hs.append(np.asarray(u, dtype=np.complex128))
    out["haar_z"] = np.asarray(zs)
    out["haar_u"] = np.asarray(hs)

    # schmidt: canonicalize + contract on seeded states
    rng = np.random.default_rng(9200)
    for n in range(2, 9):
        psi = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        psi /= np.linalg.norm(psi)
        mps = sm.canonicalize(n, psi.copy())
        out[f"schmidt_n{n}_psi"] = psi
        for b, s in enumerate(mps.L):
            out[f"schmidt_n{n}_L{b}"] = np.asarray(s, dtype=np.float64)
        out[f"schmidt_n{n}_contract"] = np.asarray(sm.contract(mps), dtype=np.complex128)

    # gate2: two qubits, a Haar gate on a random state
    for i in range(6):
        psi = rng.normal(size=4) + 1j * rng.normal(size=4)
        psi /= np.linalg.norm(psi)
        np.random.seed(9300 + i)
        u = np.asarray(random_haar(2), dtype=np.complex128)
        mps = sm.canonicalize(2, psi.copy())
        sm.apply_2q(mps, 0, u)
        out[f"gate2_{i}_psi"] = psi
        out[f"gate2_{i}_u"] = u
        out[f"gate2_{i}_L"] = np.asarray(mps.L[0], dtype=np.float64)
        out[f"gate2_{i}_contract"] = np.asarray(sm.contract(mps), dtype=np.complex128)
    # gate1: a one-qubit Haar gate (random_haar(1)) on one site of a longer
    # chain; apply_1q acts on one Gamma, which is exact for any n
    for i, (n, k) in enumerate([(3, 1), (5, 0), (5, 2), (6, 5)]):
        psi = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        psi /= np.linalg.norm(psi)
        np.random.seed(9400 + i)
        u = np.asarray(random_haar(1), dtype=np.complex128)
        mps = sm.canonicalize(n, psi.copy())
        sm.apply_1q(mps, k, u)
        out[f"gate1_{i}_nk"] = np.array([n, k])
        out[f"gate1_{i}_psi"] = psi
        out[f"gate1_{i}_u"] = u
        out[f"gate1_{i}_contract"] = np.asarray(sm.contract(mps), dtype=np.complex128)

    # proj: projection of site k onto outcome p; the prototype's project
    # contracts the sites around k without the outer Lambdas, which is exact
    # when those sites are the whole chain (n = 2, and the middle site of n = 3)
    for i, (n, k, p) in enumerate([(2, 0, 0), (2, 0, 1), (2, 1, 0), (2, 1, 1), (3, 1, 0), (3, 1, 1)]):
        psi = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        psi /= np.linalg.norm(psi)
        mps = sm.canonicalize(n, psi.copy())
        sm.project(mps, k, p)
        out[f"proj_{i}_nkp"] = np.array([n, k, p])
        out[f"proj_{i}_psi"] = psi
        for b, s in enumerate(mps.L):
            out[f"proj_{i}_L{b}"] = np.asarray(s, dtype=np.float64)
        out[f"proj_{i}_contract"] = np.asarray(sm.contract(mps), dtype=np.complex128)
    # entropy: -tr(rho log rho) of the left part (qubits 0..b) of the seeded
    # states above, by entropy.py's trace_qubit / entropy_log
    from scipy.linalg import logm
    ent = _defs("entropy.py", {"trace", "trace_qubit", "entropy_log"}, {"np": np, "logm": logm})
    for n in (4, 6, 8):
        psi = out[f"schmidt_n{n}_psi"]
        rho = np.outer(psi, psi.conj())
        red = rho
        ents = np.zeros(n - 1)
        for m in range(n, 0, -1):  # red: the density matrix of qubits 0..m-1
            if m <= n - 1:  # bond m - 1 separates qubits 0..m-1 from the rest
                ents[m - 1] = float(np.real(ent["entropy_log"](red)))
            if m > 1:
                red = ent["trace_qubit"](m, m - 1, red)
        out[f"entropy_n{n}"] = ents
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({len(out)} arrays)")


if __name__ == "__main__":
    main()
