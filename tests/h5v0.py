"""Test helper: writes HDF5 files in the structure libhdf5 produces with its
default settings, from the public HDF5 File Format Specification 3.0:
superblock version 0 (II.A.1), version-1 object headers (IV.A.1.a, messages
8-byte aligned, continuation blocks), old-style groups through a symbol
table message (IV.A.2.r) with a version-1 group B-tree (III.A.1), symbol
table nodes (III.B) of 2K = 8 entries and a local heap of names (III.D),
version-1 dataspace messages, fill value (version 2) and modification time
messages, contiguous or compact layout (version 3) and version-1 attribute
messages.

No libhdf5 is available to these tests, so files from this writer stand in
for the reference's own output files: the engine's reader must read them
as it reads its own.

tree: {name: subtree (dict) | Dataset}
"""
import struct
from dataclasses import dataclass, field

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K, INTERNAL_K = 4, 16


@dataclass
class Dataset:
    data: np.ndarray        # 1-D: int8, uint8, int32, uint64, float64, or structured {Key: i4, Value: f8}
    attrs: dict = field(default_factory=dict)  # name -> str (256-byte null-terminated string)
    compact: bool = False   # compact layout (data in the header)
    continuation: bool = False  # the attributes in a continuation block


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


def _dtype_msg(a: np.ndarray) -> bytes:
    if a.dtype.names is not None:  # compound {Key: int32 at 0, Value: float64 at 8}
        members = b""
        for name, off, sub in (("Key", 0, np.dtype(np.int32)), ("Value", 8, np.dtype(np.float64))):
            members += _pad8(name.encode() + b"\0") + struct.pack("<IB3xI4x16x", off, 0, 0)
            members += _dtype_msg(np.zeros(1, sub))
        return struct.pack("<BBBBI", 0x16, 2, 0, 0, 16) + members
    k = a.dtype.kind
    if k == "f":
        return struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 63, 0, 8, 0, 64, 52, 11, 0, 52, 1023)
    signed = 0x08 if k == "i" else 0
    n = a.dtype.itemsize
    return struct.pack("<BBBBIHH", 0x10, signed, 0, 0, n, 0, 8 * n)


def _string_type(n=256) -> bytes:
    return struct.pack("<BBBBI", 0x13, 0, 0, 0, n)


def _space_v1(dims) -> bytes:
    return struct.pack("<BBBB4x", 1, len(dims), 0, 0) + b"".join(struct.pack("<Q", d) for d in dims)


def _msg_v1(mtype: int, body: bytes) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


class Writer:
    def __init__(self):
        self.buf = bytearray(96)  # superblock, written last

    def _put(self, b: bytes, align=8) -> int:
        self.buf += b"\0" * (-len(self.buf) % align)
        at = len(self.buf)
        self.buf += b
        return at

    def _header(self, msgs: list, cont: list = None) -> int:
        """Version-1 object header; `cont` messages go to a continuation block."""
        if cont:
            block = b"".join(cont)
            at = self._put(block)
            msgs = msgs + [_msg_v1(0x10, struct.pack("<QQ", at, len(block)))]
        body = b"".join(msgs)
        n = len(msgs) + (len(cont) if cont else 0)
        return self._put(struct.pack("<BBHII4x", 1, 0, n, 1, len(body)) + body)

    def _dataset(self, ds: Dataset) -> int:
        a = np.ascontiguousarray(ds.data)
        raw = a.tobytes()
        msgs = [_msg_v1(0x01, _space_v1([len(a)])), _msg_v1(0x03, _dtype_msg(a)),
                _msg_v1(0x05, struct.pack("<BBBB", 2, 2, 0, 0)), _msg_v1(0x12, struct.pack("<B3xI", 1, 1700000000))]
        if ds.compact:
            msgs.append(_msg_v1(0x08, struct.pack("<BBH", 3, 0, len(raw)) + raw))
        else:
            at = self._put(raw) if raw else UNDEF
            msgs.append(_msg_v1(0x08, struct.pack("<BBQQ", 3, 1, at, len(raw))))
        attrs = []
        for name, value in ds.attrs.items():
            nm = name.encode() + b"\0"
            t, s = _string_type(), _space_v1([])[:8]
            v = value.encode()[:255].ljust(256, b"\0")
            attrs.append(_msg_v1(0x0C, struct.pack("<BBHHH", 1, 0, len(nm), len(t), len(s)) + _pad8(nm) + _pad8(t)
                                 + _pad8(s) + v))
        if ds.continuation:
            return self._header(msgs, attrs)
        return self._header(msgs + attrs)

    def _group(self, tree: dict, two_levels=False) -> int:
        names = sorted(tree)
        addrs = [self._write(tree[n]) for n in names]
        # local heap: "" at 0, then the names, 8-byte aligned
        seg = bytearray(8)
        offs = []
        for n in names:
            offs.append(len(seg))
            seg += _pad8(n.encode() + b"\0")
        seg_at = self._put(bytes(seg))
        heap_at = self._put(b"HEAP" + struct.pack("<B3xQQQ", 0, len(seg), UNDEF, seg_at))
        # symbol table nodes of up to 2K entries
        snods = []
        for i in range(0, max(len(names), 1), 2 * LEAF_K):
            part = list(range(i, min(i + 2 * LEAF_K, len(names))))
            ents = b"".join(struct.pack("<QQII16x", offs[k], addrs[k], 0, 0) for k in part)
            ents += b"\0" * (40 * (2 * LEAF_K - len(part)))
            snods.append((self._put(b"SNOD" + struct.pack("<BBH", 1, 0, len(part)) + ents),
                          offs[part[-1]] if part else 0))

        def node(level, children):  # children: (address, key of the largest name)
            body = struct.pack("<Q", 0)
            for addr, key in children:
                body += struct.pack("<QQ", addr, key)
            body += b"\0" * (16 * (2 * INTERNAL_K - len(children)))
            return self._put(b"TREE" + struct.pack("<BBHQQ", 0, level, len(children), UNDEF, UNDEF) + body)

        if two_levels and len(snods) > 1:
            half = (len(snods) + 1) // 2
            kids = [(node(0, snods[:half]), snods[half - 1][1]), (node(0, snods[half:]), snods[-1][1])]
            tree_at = node(1, kids)
        else:
            tree_at = node(0, snods)
        return self._header([_msg_v1(0x11, struct.pack("<QQ", tree_at, heap_at))])

    def _write(self, obj) -> int:
        if isinstance(obj, Dataset):
            return self._dataset(obj)
        return self._group({k: v for k, v in obj.items() if k != "__two_levels__"}, obj.get("__two_levels__", False))

    def write(self, path: str, tree: dict):
        root = self._write(tree)
        sb = (b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, INTERNAL_K, 0)
              + struct.pack("<QQQQ", 0, UNDEF, len(self.buf), UNDEF)
              + struct.pack("<QQII16x", 0, root, 0, 0))
        assert len(sb) == 96
        self.buf[0:96] = sb
        with open(path, "wb") as f:
            f.write(bytes(self.buf))


def write(path: str, tree: dict):
    Writer().write(path, tree)
