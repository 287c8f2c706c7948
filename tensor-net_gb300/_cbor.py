"""Minimal CBOR (RFC 8949) codec for the circuit files.

Covers the items serde_cbor 0.11 writes for tensor-net's circuit types:
unsigned / negative integers, text and byte strings, arrays, maps, floats
(half, single, double), booleans and null; tags are read and dropped.
Definite lengths are written, definite and indefinite lengths are read.

Encoding follows serde_cbor's choices: the shortest integer head, and floats
in the shortest of half / single / double that holds the value exactly (NaN
and infinities as half).  Python values map as int -> integer, float ->
float, str -> text, bytes -> byte string, list / tuple -> array, dict ->
map (insertion order), bool, None -> null.
"""
from __future__ import annotations

import math
import struct

import numpy as np


class CborError(ValueError):
    pass


# ------------------------------------------------------------------ encoding
def _head(out: bytearray, major: int, n: int):
    if n < 0:
        raise CborError("negative length")
    if n < 24:
        out.append((major << 5) | n)
    elif n < 1 << 8:
        out.append((major << 5) | 24)
        out.append(n)
    elif n < 1 << 16:
        out.append((major << 5) | 25)
        out += struct.pack(">H", n)
    elif n < 1 << 32:
        out.append((major << 5) | 26)
        out += struct.pack(">I", n)
    elif n < 1 << 64:
        out.append((major << 5) | 27)
        out += struct.pack(">Q", n)
    else:
        raise CborError("integer out of range")


def _float(out: bytearray, x: float):
    if math.isnan(x):
        out += b"\xf9\x7e\x00"
        return
    if math.isinf(x):
        out += b"\xf9\x7c\x00" if x > 0 else b"\xf9\xfc\x00"
        return
    with np.errstate(over="ignore", under="ignore"):
        f32 = np.float32(x)
        if float(f32) != x:
            out += b"\xfb" + struct.pack(">d", x)
            return
        f16 = np.float16(f32)
    if np.isfinite(f16) and float(f16) == float(f32):
        out += b"\xf9" + np.array(f16, dtype=">f2").tobytes()
    else:
        out += b"\xfa" + struct.pack(">f", float(f32))


def _enc(out: bytearray, v):
    if v is None:
        out.append(0xF6)
    elif v is True:
        out.append(0xF5)
    elif v is False:
        out.append(0xF4)
    elif isinstance(v, (int, np.integer)):
        v = int(v)
        if v >= 0:
            _head(out, 0, v)
        else:
            _head(out, 1, -1 - v)
    elif isinstance(v, (float, np.floating)):
        _float(out, float(v))
    elif isinstance(v, str):
        b = v.encode("utf-8")
        _head(out, 3, len(b))
        out += b
    elif isinstance(v, (bytes, bytearray)):
        _head(out, 2, len(v))
        out += v
    elif isinstance(v, (list, tuple)):
        _head(out, 4, len(v))
        for x in v:
            _enc(out, x)
    elif isinstance(v, dict):
        _head(out, 5, len(v))
        for k, x in v.items():
            _enc(out, k)
            _enc(out, x)
    else:
        raise CborError(f"cannot encode {type(v).__name__}")


def dumps(v) -> bytes:
    out = bytearray()
    _enc(out, v)
    return bytes(out)


# ------------------------------------------------------------------ decoding
_BREAK = object()


class _Reader:
    def __init__(self, buf: bytes):
        self.b = memoryview(buf)
        self.i = 0

    def take(self, n: int) -> bytes:
        if self.i + n > len(self.b):
            raise CborError("truncated input")
        r = bytes(self.b[self.i:self.i + n])
        self.i += n
        return r

    def arg(self, ai: int):
        if ai < 24:
            return ai
        if ai == 24:
            return self.take(1)[0]
        if ai == 25:
            return struct.unpack(">H", self.take(2))[0]
        if ai == 26:
            return struct.unpack(">I", self.take(4))[0]
        if ai == 27:
            return struct.unpack(">Q", self.take(8))[0]
        if ai == 31:
            return None  # indefinite length
        raise CborError(f"reserved additional information {ai}")

    def item(self, depth: int = 0):
        if depth > 256:
            raise CborError("nesting too deep")
        ib = self.take(1)[0]
        major, ai = ib >> 5, ib & 31
        if major == 7:
            if ai == 20:
                return False
            if ai == 21:
                return True
            if ai in (22, 23):
                return None
            if ai == 25:
                return float(np.frombuffer(self.take(2), dtype=">f2")[0])
            if ai == 26:
                return struct.unpack(">f", self.take(4))[0]
            if ai == 27:
                return struct.unpack(">d", self.take(8))[0]
            if ai == 31:
                return _BREAK
            if ai < 24:
                return None  # unassigned simple value
            if ai == 24:
                self.take(1)
                return None
            raise CborError(f"bad simple value {ai}")
        n = self.arg(ai)
        if major == 0:
            return n
        if major == 1:
            return -1 - n
        if major in (2, 3):
            if n is None:
                parts = []
                while True:
                    p = self.item(depth + 1)
                    if p is _BREAK:
                        break
                    parts.append(p.encode("utf-8") if isinstance(p, str) else p)
                raw = b"".join(parts)
            else:
                raw = self.take(n)
            return raw if major == 2 else raw.decode("utf-8")
        if major == 4:
            out = []
            while n is None or len(out) < n:
                x = self.item(depth + 1)
                if x is _BREAK:
                    if n is not None:
                        raise CborError("unexpected break")
                    break
                out.append(x)
            return out
        if major == 5:
            out = {}
            cnt = 0
            while n is None or cnt < n:
                k = self.item(depth + 1)
                if k is _BREAK:
                    if n is not None:
                        raise CborError("unexpected break")
                    break
                out[k if not isinstance(k, list) else tuple(k)] = self.item(depth + 1)
                cnt += 1
            return out
        # major 6: tag -- the tagged item stands for itself
        return self.item(depth + 1)


def loads(buf: bytes):
    r = _Reader(bytes(buf))
    v = r.item()
    if v is _BREAK:
        raise CborError("unexpected break")
    if r.i != len(r.b):
        raise CborError("trailing bytes")
    return v
