"""Circuit files: npz in the reference's save_unis / save_meas layouts
(haar.rs:54-101, lib.rs:61-147) and CBOR as serde_cbor writes the circuit
types (circuit.rs:476-517); the CBOR byte strings here follow RFC 8949's
encoding rules and serde's externally tagged enum form."""
import numpy as np
import pytest


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


# ---------------------------------------------------------------- CBOR codec (RFC 8949)
def _cb():
    from tensor_net_gb300 import _cbor
    return _cbor


@pytest.mark.parametrize("value,hexbytes", [
    (0, "00"), (23, "17"), (24, "1818"), (255, "18ff"), (256, "190100"), (500, "1901f4"),
    (65536, "1a00010000"), (2 ** 32, "1b0000000100000000"), (-1, "20"), (-24, "37"), (-25, "3818"),
    (-500, "3901f3"), (1.0, "f93c00"), (0.5, "f93800"), (-2.0, "f9c000"), (0.0, "f90000"),
    (65504.0, "f97bff"), (100000.0, "fa47c35000"), (float("inf"), "f97c00"), (float("-inf"), "f9fc00"),
    (True, "f5"), (False, "f4"), (None, "f6"), ("", "60"), ("a", "6161"), ("Rand", "6452616e64"),
    (b"\x01\x02", "420102"), ([], "80"), ([1, [2, 3]], "8201820203"), ({}, "a0"), ({"v": 1}, "a1617601"),
])
def test_cbor_encoding_follows_shortest_heads(pkg, value, hexbytes):
    cb = _cb()
    assert cb.dumps(value).hex() == hexbytes
    back = cb.loads(bytes.fromhex(hexbytes))
    assert back == value or (isinstance(value, float) and back == value)


def test_cbor_doubles_that_need_64_bits(pkg):
    import struct
    cb = _cb()
    for x in (0.1, 1.0 / 3.0, -1e-300, 6.02214076e23):
        assert cb.dumps(x) == b"\xfb" + struct.pack(">d", x)
        assert cb.loads(cb.dumps(x)) == x
    assert cb.loads(cb.dumps(float("nan"))) != cb.loads(cb.dumps(float("nan")))  # NaN
    assert cb.dumps(float("nan")).hex() == "f97e00"


def test_cbor_reads_other_encodings(pkg):
    cb = _cb()
    assert cb.loads(bytes.fromhex("9f0102ff")) == [1, 2]               # indefinite array
    assert cb.loads(bytes.fromhex("bf6161f5ff")) == {"a": True}        # indefinite map
    assert cb.loads(bytes.fromhex("5f42010241ffff")) == b"\x01\x02\xff"  # chunked bytes
    assert cb.loads(bytes.fromhex("7f6161626263ff")) == "abc"          # chunked text
    assert cb.loads(bytes.fromhex("c11a514b67b0")) == 1363896240       # a tag is dropped
    assert cb.loads(bytes.fromhex("f90001")) == 2.0 ** -24             # half subnormal
    assert cb.loads(bytes.fromhex("fa3fc00000")) == 1.5                # single
    assert cb.loads(bytes.fromhex("1800")) == 0                        # non-shortest head
    for bad in ("19", "8201", "0000", "ff", "1c"):
        with pytest.raises(cb.CborError):
            cb.loads(bytes.fromhex(bad))


def test_cbor_random_round_trip(pkg):
    cb = _cb()
    rng = np.random.default_rng(3)
    for _ in range(200):
        v = [int(rng.integers(-2 ** 62, 2 ** 62)), float(rng.standard_normal()) * 10.0 ** int(rng.integers(-30, 30)),
             {"k": [float(x) for x in rng.standard_normal(3)], "s": "x" * int(rng.integers(0, 300))},
             [[int(rng.integers(0, 2 ** 63))]]]
        assert cb.loads(cb.dumps(v)) == v


# ---------------------------------------------------------------- serde encoding of the circuit types
def test_meas_layers_bytes(pkg, tmp_path):
    from tensor_net_gb300 import circuits
    from tensor_net_gb300.gates import Meas
    f = tmp_path / "m.cbor"
    circuits.save_meas_layers(f, [[Meas.rand(3), Meas.proj(1, 1)], []])
    # [[{"Rand": 3}, {"Proj": [1, "One"]}], []]
    want = "82" + "82" + "a1" + "6452616e64" + "03" + "a1" + "6450726f6a" + "82" + "01" + "634f6e65" + "80"
    assert f.read_bytes().hex() == want
    assert circuits.load_meas_layers(f) == [[Meas.rand(3), Meas.proj(1, 1)], []]


def test_uni_layers_bytes_and_round_trip(pkg, tmp_path):
    from tensor_net_gb300 import circuits
    from tensor_net_gb300.gates import Gate, Uni
    f = tmp_path / "u.cbor"
    circuits.save_uni_layers(f, [[Uni.of_gate(Gate.H(2))]])
    assert f.read_bytes().hex() == "81" + "81" + "a1" + "6447617465" + "a1" + "6148" + "02"  # [[{"Gate": {"H": 2}}]]
    circuits.save_uni_layers(f, [[Uni.of_gate(Gate.XRot(1, 0.5))]])
    # [[{"Gate": {"XRot": [1, 0.5]}}]]
    assert f.read_bytes().hex() == "8181a16447617465" + "a1" + "6458526f74" + "82" + "01" + "f93800"
    v = circuits.load_cbor(f)
    assert v == [[{"Gate": {"XRot": [1, 0.5]}}]]
    m = np.array([[1, 0.5j], [-2, 0.1 + 0.2j]])
    circuits.save_uni_layers(f, [[Uni.mat(4, m)]])
    v = circuits.load_cbor(f)
    assert v == [[{"Mat": [4, {"v": 1, "dim": [2, 2], "data": [[1.0, 0.0], [0.0, 0.5], [-2.0, 0.0], [0.1, 0.2]]}]}]]
    raw = f.read_bytes().hex()
    assert raw.startswith("8181a1634d6174" + "82" + "04" + "a3" + "6176" + "01" + "6364696d" + "820202" + "6464617461" + "84")
    layers = [[Uni.of_gate(Gate.U(0, 0.1, 0.2, 0.3)), Uni.of_gate(Gate.CZ(1)), Uni.of_gate(Gate.Haar2(3)),
               Uni.mat(5, np.eye(4) * (1 + 2j))], [], [Uni.of_gate(Gate.ZRot(2, -1.25))]]
    circuits.save_uni_layers(f, layers)
    assert circuits.load_uni_layers(f) == layers


def test_legacy_enum_arrays_and_errors(pkg):
    from tensor_net_gb300 import circuits
    from tensor_net_gb300._cbor import CborError
    from tensor_net_gb300.gates import Gate, Meas
    assert circuits.meas_from_value(["Proj", 2, "Zero"]) == Meas.proj(2, 0)
    assert circuits.meas_from_value({"Proj": [2, 1]}) == Meas.proj(2, 1)
    assert circuits.gate_from_value(["U", 1, 0.5, 1, 2]) == Gate.U(1, 0.5, 1.0, 2.0)
    for bad in ({"Proj": [2]}, {"Foo": 1}, {"Rand": -1}, {"Proj": [1, "Two"]}, "Rand"):
        with pytest.raises(CborError):
            circuits.meas_from_value(bad)
    with pytest.raises(CborError):
        circuits.array2_from_value({"v": 2, "dim": [1, 1], "data": [[1.0, 0.0]]})
    with pytest.raises(CborError):
        circuits.array2_from_value({"v": 1, "dim": [2, 2], "data": [[1.0, 0.0]]})


def test_manifest_files_and_batch_layers(pkg, tmp_path):
    from tensor_net_gb300 import circuits
    man = circuits.MiptManifest.new(7, 8, 6, 2, [0.1, 0.25])
    assert len(man.id) == 16 and int(man.id, 16) >= 0
    assert man.meas_fname(0.1, 1) == "meas_seed=7_nqubits=8_depth=6_p=0.100000_circ=1.cbor"
    assert man.unis_fname(0) == "unis_seed=7_nqubits=8_depth=6_circ=0.cbor"
    man.save_all(tmp_path)
    back = circuits.MiptManifest.load_in(7, 8, 6, man.id, tmp_path)
    assert back == man
    assert circuits.load_cbor(tmp_path / man.manifest_fname()) == {
        "seed": 7, "nqubits": 8, "depth": 6, "num_circs": 2, "p_meas": [0.1, 0.25], "id": man.id}
    unis, meas = back.load_circuit(tmp_path, 1, 0.25)
    assert len(unis) == len(meas) == 6
    for t, (u, m) in enumerate(zip(unis, meas)):
        gk, g, mk = circuits.batch_layer(u, m)
        gk2, g2, mk2, _ = pkg.gen_layer(7, 1, t, 8, 0.25)
        np.testing.assert_array_equal(gk, gk2)
        np.testing.assert_array_equal(g, g2)
        np.testing.assert_array_equal(mk, mk2)
    with pytest.raises(ValueError):
        back.load_circuit(tmp_path, 2, 0.25)
    with pytest.raises(ValueError):
        back.load_circuit(tmp_path, 0, 0.3)


def test_npz_meas_round_trip(pkg, tmp_path):
    from tensor_net_gb300 import circuits
    from tensor_net_gb300.gates import Meas
    meas = [(0.1, [[Meas.rand(0), Meas.proj(3, 1)], []]), (0.2, [[Meas.proj(2, 0)]])]
    f = tmp_path / "meas.npz"
    circuits.save_meas(f, meas)
    z = np.load(f)
    np.testing.assert_array_equal(z["ops"], [-1, 1, 0])
    np.testing.assert_array_equal(z["layer_lens"], [2, 0, 1])
    ps, groups = circuits.load_meas(f)
    np.testing.assert_array_equal(ps, [0.1, 0.2])
    assert groups == [layers for (_, layers) in meas]


def test_cbor_fuzz_round_trip(pkg):
    """Random nested values survive dumps/loads (hypothesis, CPU only)."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from tensor_net_gb300 import _cbor
    leaves = st.one_of(st.none(), st.booleans(), st.integers(min_value=-(2 ** 64), max_value=2 ** 64 - 1),
                       st.floats(allow_nan=False), st.text(max_size=40), st.binary(max_size=40))
    values = st.recursive(leaves, lambda ch: st.one_of(st.lists(ch, max_size=6),
                                                       st.dictionaries(st.text(max_size=8), ch, max_size=6)),
                          max_leaves=30)

    @hyp.settings(max_examples=300, deadline=None)
    @hyp.given(values)
    def check(v):
        assert _cbor.loads(_cbor.dumps(v)) == v

    check()


def test_cbor_truncations_are_errors(pkg):
    """Every proper prefix of an encoding is rejected, never misread."""
    from tensor_net_gb300 import _cbor
    from tensor_net_gb300.gates import Gate, Meas, Uni
    from tensor_net_gb300 import circuits
    v = [[circuits.uni_to_value(Uni.of_gate(Gate.U(1, 0.1, 0.2, 0.3))), circuits.meas_to_value(Meas.proj(2, 1))]]
    b = _cbor.dumps(v)
    for i in range(len(b)):
        with pytest.raises(_cbor.CborError):
            _cbor.loads(b[:i])
