"""The reference's verbatim byte layout restated in Python for the tests
(crates/verbatim/src/lib.rs): each little-endian primitive is preceded by
zero bytes up to a multiple of its size counted from the start of the
stream (writer_primitive_le, lib.rs:14-27; reader_primitive_le,
lib.rs:102-119); a tag is raw bytes; a slice is a u32 length, then, when it
is not empty, zero bytes up to the element's alignment, then the elements
(write_slice, lib.rs:76-93; read_slice, lib.rs:229-258).  A state file
(crates/b3/src/mcmc.rs:251-268) starts with the tag 62 33 b3 44 and the u32
protocol version 19 (crates/b3/src/lib.rs:29)."""

import struct

STATE_TAG = bytes([0x62, 0x33, 0xB3, 0x44])
STATE_VERSION = 19

_FMT = {"u32": ("<I", 4), "u64": ("<Q", 8), "i64": ("<q", 8), "f64": ("<d", 8),
        "f32": ("<f", 4), "u16": ("<H", 2)}


class Writer:
    def __init__(self):
        self.out = bytearray()

    def _pad(self, a):
        while len(self.out) % a:
            self.out.append(0)

    def tag(self, t: bytes):
        self.out += t

    def prim(self, kind, v):
        fmt, size = _FMT[kind]
        self._pad(size)
        self.out += struct.pack(fmt, v)

    def u128(self, v: int):
        self._pad(16)
        self.out += v.to_bytes(16, "little")

    def slice(self, kind, values):
        fmt, size = _FMT[kind]
        self.prim("u32", len(values))
        if values:
            self._pad(size)
        for v in values:
            self.out += struct.pack(fmt, v)


class Reader:
    def __init__(self, data: bytes):
        self.data = bytes(data)
        self.at = 0

    def _take(self, n):
        if self.at + n > len(self.data):
            raise EOFError("state ends early")
        b = self.data[self.at:self.at + n]
        self.at += n
        return b

    def _skip(self, a):
        r = self.at % a
        if r:
            self._take(a - r)

    def tag(self, n):
        return self._take(n)

    def prim(self, kind):
        fmt, size = _FMT[kind]
        self._skip(size)
        return struct.unpack(fmt, self._take(size))[0]

    def u128(self):
        self._skip(16)
        return int.from_bytes(self._take(16), "little")

    def slice(self, kind):
        fmt, size = _FMT[kind]
        n = self.prim("u32")
        if n:
            self._skip(size)
        return [struct.unpack(fmt, self._take(size))[0] for _ in range(n)]

    def left(self):
        return len(self.data) - self.at
