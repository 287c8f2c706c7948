"""The committed golden trajectories: the generator reproduces their inputs
bit for bit and the FP64 oracle reproduces their results (a pin of the oracle
across numpy / LAPACK builds).  The GPU comparison is in test_gpu_golden.py."""
import numpy as np

from golden_cases import load


def test_generator_reproduces_golden_inputs(pkg):
    for c in load():
        for t, (gk, g, mk, us) in enumerate(c["layers"]):
            gk2, g2, mk2, us2 = pkg.gen_layer(c["seed"], c["traj"], t, c["n"], c["p"])
            np.testing.assert_array_equal(gk, gk2)
            np.testing.assert_array_equal(g, g2)
            np.testing.assert_array_equal(mk, mk2)
            np.testing.assert_array_equal(us, us2)


def test_oracle_reproduces_golden_results(ref):
    for c in load():
        m = ref.MPS(c["n"], ref.Trunc.both(c["chi"], c["cutoff"]))
        for t, layer in enumerate(c["layers"]):
            rec = ref.apply_bilayer(m, *layer)
            assert [r[:2] for r in rec] == [r[:2] for r in c["recs"][t]], (c["name"], t)
            np.testing.assert_allclose([r[2] for r in rec], [r[2] for r in c["recs"][t]], atol=1e-12)
            assert abs(m.entropy_vn(c["n"] // 2 - 1) - c["entropy"][t]) < 1e-12
        for b in range(c["n"] - 1):
            np.testing.assert_allclose(m.svals[b], c["svals"][b], rtol=1e-10, atol=1e-14)
