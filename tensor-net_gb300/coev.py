"""Multi-chi coevolution replay (workspace/src/haar_coev_probs.rs:34-80).

For every run, one trajectory of the circuit is sampled without truncation
(BondDim None) -- its measurement outcomes are recorded -- and the same
circuit is replayed once per chi_max with every measurement post-selected on
the recorded outcome (Meas::Proj), recording the Born probability of each
outcome (prob_data[run, chi, measurement]; the sampled trajectory's own
probabilities come last, as in the reference).

GPU-native layout: the samplers of all runs are one batch, the replays of all
runs and chi values another; both advance one brickwork layer per launch, the
replays right after the samplers, taking that layer's outcomes as
post-selections.  The circuit (gates and measurement sites) is shared by all
runs; only the outcome uniforms differ between runs.
"""
from __future__ import annotations

import numpy as np

from .batch import Batch
from .inputs import gen_layer
from .mps import Trunc

# chi_max values of the reference driver (haar_coev_probs.rs:16-22); None = no truncation
REFERENCE_BONDS = (4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 56, 64, 72, None)


def run_uniforms(seed: int, run: int, layer: int, count: int) -> np.ndarray:
    """Outcome uniforms of one run's layer (independent of the circuit)."""
    rng = np.random.default_rng([seed, 0x636F6576, run, layer])
    return rng.random(count)


def run_coevolution(n: int, depth: int, p: float, runs: int, seed: int, circuit: int = 0,
                    bonds=REFERENCE_BONDS, precision: str = "f64"):
    """Coevolution of the seeded brickwork circuit ``gen_layer(seed, circuit,
    t, n, p)``, t < depth.  Returns dict(outcomes[runs, M], probs[runs,
    len(bonds), M], sites[M, 2] (layer, qubit)) with M the circuit's number of
    measurements; the last entry of `bonds` must be None (the sampled
    trajectories)."""
    layers = [gen_layer(seed, circuit, t, n, p)[:3] for t in range(depth)]
    return run_coevolution_layers(n, layers, runs, seed, bonds, precision)


def run_coevolution_files(manifest_path, circ: int, p: float, runs: int, seed: int,
                          bonds=REFERENCE_BONDS, precision: str = "f64"):
    """The reference driver's inputs (haar_coev_probs.rs:96-140): a
    ``MiptManifest`` CBOR file, a circuit number and a p of the manifest; the
    unitary and measurement CBOR files are read from the manifest's folder."""
    import os

    from .circuits import MiptManifest, batch_layer
    man = MiptManifest.load(manifest_path)
    unis, meas = man.load_circuit(os.path.dirname(os.path.abspath(manifest_path)), circ, p)
    if len(unis) != len(meas):
        raise ValueError("unitary and measurement files differ in depth")
    layers = [batch_layer(u, m) for u, m in zip(unis, meas)]
    return run_coevolution_layers(man.nqubits, layers, runs, seed, bonds, precision)


def run_coevolution_layers(n: int, layers, runs: int, seed: int, bonds=REFERENCE_BONDS,
                           precision: str = "f64"):
    """Coevolution over explicit layers ``[(gate_ks, gates[ng, 4, 4], meas_ks)]``;
    run r draws its outcome uniforms from ``run_uniforms(seed, r, t, .)``."""
    assert bonds[-1] is None, "the untruncated sampler comes last"
    chis = [c for c in bonds if c is not None]
    sampler = Batch([n] * runs, [Trunc.none()] * runs, precision)
    replay = Batch([n] * (runs * len(chis)), [Trunc.const(c) for _ in range(runs) for c in chis], precision)
    s_ids = list(range(runs))
    r_ids = list(range(runs * len(chis)))
    outcomes, probs, sites = [], [], []
    for t, (gk, g, mk) in enumerate(layers):
        # the surviving targets in the order the layer measures them (mps.rs:2214-2220),
        # so that outcome j of the sampler is post-selection j of the replays
        mk = np.unique(np.asarray(mk, np.int64)[np.asarray(mk, np.int64) < n]).astype(np.uint32)
        slayers = [(gk, g, mk, run_uniforms(seed, r, t, len(mk))) for r in range(runs)]
        recs, _ = sampler.step(s_ids, slayers)
        post = [np.array([o for (_, o, _) in recs[r]], np.int32) for r in range(runs)]
        rlayers = [(gk, g, mk, np.zeros(len(mk))) for r in range(runs) for _ in chis]
        rposts = [post[r] for r in range(runs) for _ in chis]
        rrecs, _ = replay.step(r_ids, rlayers, posts=rposts)
        sites += [(t, int(k)) for k in mk]
        outcomes.append(np.array([[o for (_, o, _) in recs[r]] for r in range(runs)], np.int32).reshape(runs, -1))
        pr = np.zeros((runs, len(bonds), len(mk)))
        for r in range(runs):
            for ci in range(len(chis)):
                pr[r, ci] = [q for (_, _, q) in rrecs[r * len(chis) + ci]]
            pr[r, -1] = [q for (_, _, q) in recs[r]]
        probs.append(pr)
    status = (sampler.device_status(), replay.device_status())
    sampler.close()
    replay.close()
    return dict(outcomes=np.concatenate(outcomes, axis=1), probs=np.concatenate(probs, axis=2),
                sites=np.array(sites, np.int32).reshape(-1, 2), device_status=status)
