"""Circuit files of the reference, read and written on the host.

npz (workspace/lib/haar.rs:54-101, `save_unis` / `load_unis`): arrays `depth`
(uint32, layer of each gate), `targs` (uint32, left qubit of each gate) and
`mats` (complex128, one 4x4 matrix per gate), gates of a layer contiguous.
Loading groups consecutive entries with equal depth into one layer, as
`load_unis` does (a depth with no gate yields no layer).  Measurement layers
in npz: `save_meas` / `load_meas` (workspace/lib/lib.rs:61-147).

CBOR (circuit.rs:476-517, `save_cbor` / `load_cbor` over serde_cbor 0.11):
`Vec<Vec<Uni>>` unitary files, `Vec<Vec<Meas>>` measurement files and the
`MiptManifest` that names them (workspace/lib/haar.rs:211-320), in serde's
encoding of those types (externally tagged enums, ndarray's {v, dim, data}
struct, num-complex's (re, im) tuples, structs as maps keyed by field name).

The layers feed `MPS.apply_bilayer(_ops)`, `Batch.step` or `tn_batch_step`.
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass

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


# ---------------------------------------------------------------- npz: measurements
def save_meas(path, meas):
    """workspace/lib/lib.rs:61-105 (``save_meas``): ``meas`` is a list of
    ``(p, layers)`` with ``layers[t]`` a list of ``Meas``; arrays ``pvals``
    (float64, one per layer), ``layer_lens`` (uint32), ``targs`` (uint32) and
    ``ops`` (int32: -1 = Rand, 0 / 1 = post-selected outcome)."""
    pvals, lens, targs, ops = [], [], [], []
    for p, layers in meas:
        for layer in layers:
            for m in layer:
                targs.append(m.k)
                ops.append(-1 if m.is_rand() else int(m.outcome))
            pvals.append(float(p))
            lens.append(len(layer))
    np.savez(path, pvals=np.asarray(pvals, np.float64), layer_lens=np.asarray(lens, np.uint32),
             targs=np.asarray(targs, np.uint32), ops=np.asarray(ops, np.int32))


def load_meas(path):
    """workspace/lib/lib.rs:107-147 (``load_meas``): returns ``(p[np], [layers
    per p])``; consecutive layers with equal ``pvals`` form one group."""
    from .gates import Meas
    z = np.load(path)
    pvals = np.asarray(z["pvals"], np.float64).reshape(-1)
    lens = np.asarray(z["layer_lens"]).astype(np.int64).reshape(-1)
    targs = np.asarray(z["targs"]).astype(np.int64).reshape(-1)
    ops = np.asarray(z["ops"]).astype(np.int64).reshape(-1)
    if len(pvals) != len(lens) or len(targs) != len(ops) or int(lens.sum()) > len(targs):
        raise ValueError("operations list ended unexpectedly")
    ps, groups, j = [], [], 0
    for i in range(len(pvals)):
        if i == 0 or pvals[i] != pvals[i - 1]:
            ps.append(float(pvals[i]))
            groups.append([])
        layer = []
        for _ in range(int(lens[i])):
            t, o = int(targs[j]), int(ops[j])
            layer.append(Meas.proj(t, o) if o in (0, 1) else Meas.rand(t))
            j += 1
        groups[-1].append(layer)
    return np.asarray(ps, np.float64), groups


# ---------------------------------------------------------------- CBOR (serde_cbor)
# serde's externally tagged enums as serde_cbor 0.11 writes them: a unit
# variant is its name; a newtype variant {name: value}; a tuple variant
# {name: [fields]}.  The legacy array form [name, fields...] is also read.
_GATE_ARITY = {"U": 4, "XRot": 2, "ZRot": 2, "H": 1, "X": 1, "Z": 1, "S": 1, "SInv": 1, "CX": 1,
               "CXRev": 1, "CZ": 1, "Haar2": 1}
_UNI_ARITY = {"Gate": 1, "Mat": 2}
_MEAS_ARITY = {"Rand": 1, "Proj": 2}
_OUTCOMES = ("Zero", "One")


def _tag(name, fields):
    return {name: fields[0] if len(fields) == 1 else list(fields)}


def _untag(v, arity, what):
    from ._cbor import CborError
    if isinstance(v, dict) and len(v) == 1:
        (name, payload), = v.items()
        if name not in arity:
            raise CborError(f"unknown {what} variant {name!r}")
        if arity[name] == 1:
            return name, [payload]
        if not isinstance(payload, list) or len(payload) != arity[name]:
            raise CborError(f"{what}::{name} needs {arity[name]} fields")
        return name, payload
    if isinstance(v, list) and v and isinstance(v[0], str) and v[0] in arity:
        if len(v) - 1 != arity[v[0]]:
            raise CborError(f"{what}::{v[0]} needs {arity[v[0]]} fields")
        return v[0], v[1:]
    raise CborError(f"not a {what} value: {v!r}")


def _usize(x):
    from ._cbor import CborError
    if not isinstance(x, int) or isinstance(x, bool) or x < 0:
        raise CborError(f"expected an unsigned integer, got {x!r}")
    return x


def _num(x):
    from ._cbor import CborError
    if isinstance(x, bool) or not isinstance(x, (int, float)):
        raise CborError(f"expected a number, got {x!r}")
    return float(x)


def array2_to_value(m):
    """ndarray's serde form of an ``Array2<C64>`` (format version 1): struct
    {v, dim, data}, data in row-major order, each entry num-complex's
    ``(re, im)`` tuple."""
    a = np.asarray(m, dtype=np.complex128)
    if a.ndim != 2:
        raise ValueError("expected a 2-D matrix")
    return {"v": 1, "dim": [int(a.shape[0]), int(a.shape[1])],
            "data": [[float(z.real), float(z.imag)] for z in a.reshape(-1)]}


def array2_from_value(v):
    from ._cbor import CborError
    if isinstance(v, list) and len(v) == 3:
        v = {"v": v[0], "dim": v[1], "data": v[2]}
    if not isinstance(v, dict) or set(v) != {"v", "dim", "data"}:
        raise CborError("not an ndarray value")
    if v["v"] != 1:
        raise CborError(f"unknown ndarray format version {v['v']!r}")
    dim = v["dim"]
    if not isinstance(dim, list) or len(dim) != 2:
        raise CborError("Array2 needs two dimensions")
    r, c = _usize(dim[0]), _usize(dim[1])
    data = v["data"]
    if not isinstance(data, list) or len(data) != r * c:
        raise CborError("ndarray data length does not match its shape")
    out = np.empty(r * c, dtype=np.complex128)
    for i, z in enumerate(data):
        if not isinstance(z, list) or len(z) != 2:
            raise CborError("complex entries are (re, im) pairs")
        out[i] = complex(_num(z[0]), _num(z[1]))
    return out.reshape(r, c)


def gate_to_value(g):
    """``Gate`` (gate.rs:25-57)."""
    return _tag(g.kind, [g.k, *g.params])


def gate_from_value(v):
    from .gates import Gate
    name, f = _untag(v, _GATE_ARITY, "Gate")
    return Gate(name, _usize(f[0]), tuple(_num(x) for x in f[1:]))


def uni_to_value(u):
    """``Uni`` (circuit.rs:210-216)."""
    if u.is_gate():
        return {"Gate": gate_to_value(u.gate)}
    return {"Mat": [int(u.k), array2_to_value(u.matrix)]}


def uni_from_value(v):
    from .gates import Uni
    name, f = _untag(v, _UNI_ARITY, "Uni")
    if name == "Gate":
        return Uni.of_gate(gate_from_value(f[0]))
    return Uni.mat(_usize(f[0]), array2_from_value(f[1]))


def meas_to_value(m):
    """``Meas`` (circuit.rs:345-348), ``Outcome`` as its variant name (circuit.rs:73-78)."""
    if m.is_rand():
        return {"Rand": int(m.k)}
    return {"Proj": [int(m.k), _OUTCOMES[m.outcome]]}


def meas_from_value(v):
    from ._cbor import CborError
    from .gates import Meas
    name, f = _untag(v, _MEAS_ARITY, "Meas")
    if name == "Rand":
        return Meas.rand(_usize(f[0]))
    o = f[1]
    if isinstance(o, str) and o in _OUTCOMES:
        o = _OUTCOMES.index(o)
    elif isinstance(o, dict) and len(o) == 1 and next(iter(o)) in _OUTCOMES:
        o = _OUTCOMES.index(next(iter(o)))
    elif not (isinstance(o, int) and o in (0, 1)):
        raise CborError(f"not an Outcome: {o!r}")
    return Meas.proj(_usize(f[0]), o)


def save_cbor(value, path):
    """``save_cbor`` (circuit.rs:476-497): CBOR of a plain value, overwriting ``path``."""
    from . import _cbor
    with open(path, "wb") as fh:
        fh.write(_cbor.dumps(value))


def load_cbor(path):
    """``load_cbor`` (circuit.rs:499-517)."""
    from . import _cbor
    with open(path, "rb") as fh:
        return _cbor.loads(fh.read())


def save_uni_layers(path, layers):
    """``Vec<UniSeq>`` (one list of ``Uni`` per layer) as serde_cbor writes it."""
    save_cbor([[uni_to_value(u) for u in layer] for layer in layers], path)


def load_uni_layers(path):
    from ._cbor import CborError
    v = load_cbor(path)
    if not isinstance(v, list) or not all(isinstance(x, list) for x in v):
        raise CborError("expected a list of unitary layers")
    return [[uni_from_value(u) for u in layer] for layer in v]


def save_meas_layers(path, layers):
    """``Vec<MeasSeq>`` (one list of ``Meas`` per layer)."""
    save_cbor([[meas_to_value(m) for m in layer] for layer in layers], path)


def load_meas_layers(path):
    from ._cbor import CborError
    v = load_cbor(path)
    if not isinstance(v, list) or not all(isinstance(x, list) for x in v):
        raise CborError("expected a list of measurement layers")
    return [[meas_from_value(m) for m in layer] for layer in v]


def uni_layer_from_arrays(gate_ks, gates):
    """A brickwork layer ``(gate_ks, gates[ng, 4, 4])`` as ``Uni::Mat`` values,
    the form ``haar_layer`` produces (circuit.rs:556-563)."""
    from .gates import Uni
    g = np.asarray(gates, dtype=np.complex128).reshape(-1, 4, 4)
    return [Uni.mat(int(k), m) for k, m in zip(np.asarray(gate_ks).reshape(-1), g)]


def batch_layer(unis, meas):
    """``(gate_ks, gates[ng, 4, 4], meas_ks)`` for ``Batch.step`` /
    ``MPS.apply_bilayer`` from a ``Uni`` layer and a ``Meas`` layer.  Only
    two-qubit elements (4x4 ``Mat`` or a two-qubit ``Gate``) and ``Rand``
    measurements map onto these inputs; one-qubit elements run through
    ``MPS.apply_bilayer_ops`` and post-selections through the ``posts`` of
    ``Batch.step``."""
    ks, gs = [], []
    for u in unis:
        if u.is_gate():
            if not u.gate.is_q2() or u.gate.kind == "Haar2":
                raise ValueError(f"{u.gate.kind} is not a fixed two-qubit matrix; use MPS.apply_bilayer_ops")
            k, m = u.gate.into_matrix()
        else:
            if np.shape(u.matrix) != (4, 4):
                raise ValueError("only 4x4 matrices map onto the batched inputs")
            k, m = u.k, u.matrix
        ks.append(k)
        gs.append(m)
    mk = []
    for m in meas:
        if not m.is_rand():
            raise ValueError("post-selected measurements go through Batch.step(posts=...)")
        mk.append(m.k)
    return (np.asarray(ks, np.uint32), np.asarray(gs, np.complex128).reshape(-1, 4, 4),
            np.asarray(mk, np.uint32))


# ---------------------------------------------------------------- circuit manifests
@dataclass(frozen=True)
class MiptManifest:
    """``MiptManifest`` (workspace/lib/haar.rs:211-320): a batch of generated
    circuits, with the reference's file names.  ``id`` is 16 hex digits; the
    reference derives it from Rust's SipHash and a ChaCha12 draw, which this
    module does not reproduce (``new`` uses a BLAKE2 hash of the same fields);
    a manifest read from a file keeps the id it was written with."""

    seed: int
    nqubits: int
    depth: int
    num_circs: int
    p_meas: tuple
    id: str

    @staticmethod
    def new(seed: int, nqubits: int, depth: int, num_circs: int, p_meas):
        import hashlib
        ps = tuple(float(p) for p in p_meas)
        h = hashlib.blake2b(digest_size=8)
        for x in (seed, nqubits, depth, num_circs):
            h.update(int(x).to_bytes(8, "little"))
        for p in ps:
            h.update(struct.pack("<d", p))
        return MiptManifest(int(seed), int(nqubits), int(depth), int(num_circs), ps, h.hexdigest())

    def unis_fname(self, circ: int) -> str:
        return f"unis_seed={self.seed}_nqubits={self.nqubits}_depth={self.depth}_circ={circ}.cbor"

    def meas_fname(self, p: float, circ: int) -> str:
        return f"meas_seed={self.seed}_nqubits={self.nqubits}_depth={self.depth}_p={p:.6f}_circ={circ}.cbor"

    @staticmethod
    def manifest_fmt(seed: int, nqubits: int, depth: int, id: str) -> str:
        return f"manifest_seed={seed}_nqubits={nqubits}_depth={depth}_id={id}.cbor"

    def manifest_fname(self) -> str:
        return self.manifest_fmt(self.seed, self.nqubits, self.depth, self.id)

    def to_value(self):
        return {"seed": self.seed, "nqubits": self.nqubits, "depth": self.depth, "num_circs": self.num_circs,
                "p_meas": [float(p) for p in self.p_meas], "id": self.id}

    @staticmethod
    def from_value(v):
        from ._cbor import CborError
        keys = ("seed", "nqubits", "depth", "num_circs", "p_meas", "id")
        if isinstance(v, list) and len(v) == 6:
            v = dict(zip(keys, v))
        if not isinstance(v, dict) or not all(k in v for k in keys):
            raise CborError("not a MiptManifest value")
        if not isinstance(v["p_meas"], list) or not isinstance(v["id"], str):
            raise CborError("bad MiptManifest fields")
        return MiptManifest(_usize(v["seed"]), _usize(v["nqubits"]), _usize(v["depth"]), _usize(v["num_circs"]),
                            tuple(_num(p) for p in v["p_meas"]), v["id"])

    def save(self, outdir):
        save_cbor(self.to_value(), os.path.join(outdir, self.manifest_fname()))

    @staticmethod
    def load(path):
        return MiptManifest.from_value(load_cbor(path))

    @staticmethod
    def load_in(seed: int, nqubits: int, depth: int, id: str, indir):
        return MiptManifest.load(os.path.join(indir, MiptManifest.manifest_fmt(seed, nqubits, depth, id)))

    def save_all(self, outdir):
        """``save_all`` (haar.rs:277-299): per circuit one unitary file (Haar
        brickwork, ``Uni::Mat``) and one measurement file per p (``Meas::Rand``
        sites of ``uniform_meas``), then the manifest.  The layers come from
        this package's seeded generator (``gen_layer(seed, circ, t, n, p)``),
        not from the reference's ``StdRng`` stream."""
        from .gates import Meas
        from .inputs import gen_layer
        for circ in range(self.num_circs):
            layers = [gen_layer(self.seed, circ, t, self.nqubits, 0.0) for t in range(self.depth)]
            save_uni_layers(os.path.join(outdir, self.unis_fname(circ)),
                            [uni_layer_from_arrays(gk, g) for (gk, g, _, _) in layers])
            for p in self.p_meas:
                meas = [[Meas.rand(int(k)) for k in gen_layer(self.seed, circ, t, self.nqubits, p)[2]]
                        for t in range(self.depth)]
                save_meas_layers(os.path.join(outdir, self.meas_fname(p, circ)), meas)
        self.save(outdir)

    def load_circuit(self, indir, circ: int, p: float):
        """The unitary and measurement layers of circuit ``circ`` at ``p``
        (haar_coev_probs.rs:133-140)."""
        if circ >= self.num_circs:
            raise ValueError(f"invalid circuit number {circ} for {self.num_circs} total circuits")
        if float(p) not in self.p_meas:
            raise ValueError(f"invalid p value {p:.6f} for batch values {list(self.p_meas)}")
        unis = load_uni_layers(os.path.join(indir, self.unis_fname(circ)))
        meas = load_meas_layers(os.path.join(indir, self.meas_fname(p, circ)))
        return unis, meas
