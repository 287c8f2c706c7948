"""npz circuit files in the reference's save_unis layout (haar.rs:54-101)."""
import numpy as np


def test_npz_round_trip_and_reference_layout(pkg, tmp_path):
    from tensor_net_gb300 import circuits
    n, depth = 8, 5
    layers = [pkg.gen_layer(4, 0, t, n, 0.0)[:2] for t in range(depth)]
    f = tmp_path / "unis.npz"
    circuits.save_unis(f, layers)
    z = np.load(f)
    assert z["depth"].dtype == np.uint32 and z["targs"].dtype == np.uint32 and z["mats"].dtype == np.complex128
    assert z["mats"].shape == (sum(len(L[0]) for L in layers), 4, 4)
    back = circuits.load_unis(f)
    assert len(back) == depth
    for (gk, g), (gk2, g2) in zip(layers, back):
        np.testing.assert_array_equal(gk, gk2)
        np.testing.assert_array_equal(g, g2)


def test_load_groups_consecutive_depths_like_load_unis(tmp_path):
    from tensor_net_gb300 import circuits
    eye = np.eye(4, dtype=np.complex128)
    f = tmp_path / "c.npz"
    # depth 1 has no gate: the reference's chunk_by yields no layer for it
    np.savez(f, depth=np.array([0, 0, 2], np.uint32), targs=np.array([0, 2, 1], np.uint32),
             mats=np.stack([eye, 2 * eye, 3 * eye]))
    layers = circuits.load_unis(f)
    assert [list(L[0]) for L in layers] == [[0, 2], [1]]
    assert layers[1][1][0][0, 0] == 3
