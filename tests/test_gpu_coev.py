"""Batched post-selection (Meas::Proj, mps.rs:2236-2242) and the multi-chi
coevolution replay (haar_coev_probs.rs:34-80) against the FP64 oracle on the
same circuit, uniforms and recorded outcomes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_post_selection_matches_oracle(pkg, ref):
    """Trajectory 0 post-selects every measurement on the outcome a sampled
    oracle trajectory drew; trajectory 1 post-selects every other one and
    samples the rest with the same uniforms.  Both must reproduce the sampled
    trajectory's records and entropies (post-selection on an outcome that
    occurred never has zero probability)."""
    n, chi = 8, 8
    b = pkg.Batch([n, n], [pkg.Trunc.const(chi)] * 2, "f64")
    samp = ref.MPS(n, ref.Trunc.const(chi))
    for t in range(8):
        gk, g, mk, us = pkg.gen_layer(3, 0, t, n, 0.4)
        want = ref.apply_bilayer(samp, gk, g, mk, us)
        outs = np.array([o for (_, o, _) in want], np.int32)
        posts = [outs, np.array([o if j % 2 == 0 else -1 for j, o in enumerate(outs)], np.int32)]
        recs, ents = b.step([0, 1], [(gk, g, mk, us)] * 2, posts=posts)
        for rec in recs:
            assert [x[:2] for x in rec] == [x[:2] for x in want]
            np.testing.assert_allclose([x[2] for x in rec], [x[2] for x in want], atol=1e-9)
        np.testing.assert_allclose(ents, [samp.entropy_vn(n // 2 - 1)] * 2, atol=1e-9)
    assert b.device_status() == 0


def test_coevolution_replay_matches_oracle(pkg, ref):
    n, depth, p, runs, seed = 8, 6, 0.3, 2, 21
    bonds = (4, 8, None)
    out = pkg.run_coevolution(n, depth, p, runs, seed, bonds=bonds, precision="f64")
    assert out["device_status"] == (0, 0)
    M = out["sites"].shape[0]
    assert out["outcomes"].shape == (runs, M) and out["probs"].shape == (runs, len(bonds), M)
    from tensor_net_gb300.coev import run_uniforms
    for r in range(runs):
        samp = ref.MPS(n, ref.Trunc.none())
        reps = [ref.MPS(n, ref.Trunc.const(c)) for c in bonds[:-1]]
        col = 0
        for t in range(depth):
            gk, g, mk, _ = pkg.gen_layer(seed, 0, t, n, p)
            us = run_uniforms(seed, r, t, len(mk))
            rec = ref.apply_bilayer(samp, gk, g, mk, us)
            outs = [o for (_, o, _) in rec]
            np.testing.assert_array_equal(out["outcomes"][r, col:col + len(mk)], outs)
            np.testing.assert_allclose(out["probs"][r, -1, col:col + len(mk)], [q for (_, _, q) in rec], atol=1e-9)
            for ci, m in enumerate(reps):
                for k, op in zip(gk, g):
                    m.apply_unitary2(int(k), op)
                rr = m.apply_meas_prob_layer(mk, np.zeros(len(mk)), posts=outs)
                np.testing.assert_allclose(out["probs"][r, ci, col:col + len(mk)], [q for (_, _, q) in rr],
                                           atol=1e-9)
            col += len(mk)


def test_coevolution_from_cbor_circuit_files(pkg, tmp_path):
    """The reference driver's inputs (a MiptManifest and its CBOR unitary /
    measurement files) give the same coevolution as the same circuit fed as
    arrays."""
    from tensor_net_gb300 import circuits
    from tensor_net_gb300.coev import run_coevolution, run_coevolution_files
    # circuit seed 9 (the manifest's) = the uniforms' seed of run_coevolution
    man = circuits.MiptManifest.new(9, 8, 6, 1, [0.2])
    man.save_all(tmp_path)
    a = run_coevolution_files(tmp_path / man.manifest_fname(), 0, 0.2, 2, 9, bonds=(4, 8, None))
    b = run_coevolution(8, 6, 0.2, 2, 9, circuit=0, bonds=(4, 8, None))
    np.testing.assert_array_equal(a["sites"], b["sites"])
    np.testing.assert_array_equal(a["outcomes"], b["outcomes"])
    np.testing.assert_array_equal(a["probs"], b["probs"])
    assert a["device_status"] == (0, 0)


@pytest.mark.parametrize("prec", ["f64", "df"])
def test_cbor_circuit_files_through_the_gpu_match_the_oracle(pkg, ref, tmp_path, prec):
    """A seeded Haar brickwork circuit written to the reference's CBOR
    formats (Vec<Vec<Uni>> and Vec<Vec<Meas>>, circuit.rs:479-517), read back
    and run through the GPU single-state API, against the FP64 oracle fed the
    original arrays: outcomes, probabilities and per-layer entropies."""
    from tensor_net_gb300 import circuits
    from tensor_net_gb300.gates import Meas
    n, chi, depth, p, seed = 10, 16, 8, 0.25, 33
    layers = pkg.gen_trajectory(seed, 0, n, depth, p)
    circuits.save_uni_layers(tmp_path / "unis.cbor",
                             [circuits.uni_layer_from_arrays(gk, g) for (gk, g, _, _) in layers])
    circuits.save_meas_layers(tmp_path / "meas.cbor", [[Meas.rand(int(k)) for k in mk] for (_, _, mk, _) in layers])
    unis = circuits.load_uni_layers(tmp_path / "unis.cbor")
    meas = circuits.load_meas_layers(tmp_path / "meas.cbor")
    assert len(unis) == len(meas) == depth
    g = pkg.MPS.new_qubits(n, pkg.Trunc.both(chi, 1e-12), prec)
    r = ref.MPS(n, ref.Trunc.both(chi, 1e-12))
    for (gk, gs, mk, us), ul, ml in zip(layers, unis, meas):
        outs, probs = g.apply_bilayer_ops(ul, ml, us)
        rec = ref.apply_bilayer(r, gk, gs, mk, us)
        assert [(m.k, m.outcome) for m in outs] == [(k, o) for (k, o, _) in rec]
        np.testing.assert_allclose([q for (_, q) in probs], [q for (_, _, q) in rec], atol=1e-9)
        assert abs(g.entropy_vn(n // 2 - 1) - r.entropy_vn(n // 2 - 1)) < 1e-9
    assert g.device_status() == 0
