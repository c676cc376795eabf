"""HDF5 result files without libhdf5 (qec_pf_wang_landau_gb300/csrc/wlg_h5.*).

No libhdf5 or h5py is available to these tests, so the writer follows the
public HDF5 File Format Specification and is checked three ways: its
checksum against lookup3's published test vectors, a round trip through the
engine's own reader, and an independent parse of the superblock, object
headers and links here (structure, versions, checksums).
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def engine():
    import qec_pf_wang_landau_gb300 as wlg
    wlg.build()
    return wlg


def test_lookup3_published_vectors(engine):
    L = engine.lib()
    h = lambda s, init: L.wlg_h5_lookup3(s, len(s), init)
    assert h(b"", 0) == 0xDEADBEEF
    assert h(b"Four score and seven years ago", 0) == 0x17770551
    assert h(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.fixture(scope="module")
def written(engine, tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("h5")
    exe = d / "h5_write"
    pkg = os.path.join(ROOT, "qec_pf_wang_landau_gb300")
    subprocess.run([cxx, "-std=c++20", "-O1", os.path.join(ROOT, "tests", "csrc", "h5_write.cpp"), "-o", str(exe),
                    "-L" + pkg, "-lwlg", "-Wl,-rpath," + pkg], check=True)
    path = d / "f.h5"
    subprocess.run([str(exe), str(path)], check=True)
    return str(path)


def test_round_trip_through_reader(engine, written):
    groups, dsets = engine.h5_list(written)
    assert groups == ["0", "Histogram", "Interaction", "Lattice"] and dsets == []
    assert engine.h5_list(written, "Lattice/0")[0] == ["-8", "12"]
    assert engine.h5_read(written, "Histogram/0/Histogram").tolist() == [0, 1, 1, 0, 1]
    assert engine.h5_read(written, "Histogram/0/Histogram").dtype == np.dtype("<u8")
    assert engine.h5_read(written, "Interaction/0/Interaction").tolist() == [1, -1, 1, 1, -1, 1, 1, 1]
    assert engine.h5_read(written, "Lattice/0/12/Lattice").tolist() == [-1, 1, -1, 1]
    kv = engine.h5_read(written, "0/12345/Thu_Dec__3_18:00:00_2026/log_g")
    assert kv["Key"].tolist() == [-8, -4, 0] and kv["Value"].tolist() == [0.5, 1.25, 2.75]
    assert engine.h5_attribute(written, "0/12345/Thu_Dec__3_18:00:00_2026/log_g", "CodeVersion") == "wlg test 1"


def _parse(engine, path):
    """Independent walk: superblock v2, v2 object headers, link messages."""
    b = open(path, "rb").read()
    lk = lambda data: engine.lib().wlg_h5_lookup3(data, len(data), 0)
    assert b[:8] == b"\x89HDF\r\n\x1a\n" and b[8] == 2 and b[9] == 8 and b[10] == 8
    base, ext, eof, root = struct.unpack_from("<QQQQ", b, 12)
    assert base == 0 and ext == 2 ** 64 - 1 and eof == len(b)
    assert struct.unpack_from("<I", b, 44)[0] == lk(b[:44])

    def obj(addr):
        assert b[addr:addr + 4] == b"OHDR" and b[addr + 4] == 2
        flags = b[addr + 5]
        assert flags & 3 == 2  # 4-byte chunk size
        size = struct.unpack_from("<I", b, addr + 6)[0]
        end = addr + 10 + size
        assert struct.unpack_from("<I", b, end)[0] == lk(b[addr:end])
        msgs, p = [], addr + 10
        while p + 4 <= end:
            t, n, f = struct.unpack_from("<BHB", b, p)
            msgs.append((t, b[p + 4:p + 4 + n]))
            p += 4 + n
        assert p == end
        return msgs

    def walk(addr, depth=0):
        msgs = obj(addr)
        types = [t for t, _ in msgs]
        if 8 in types:  # dataset: dataspace, datatype, fill value, layout
            assert types[:4] == [1, 3, 5, 8]
            layout = dict(msgs)[8]
            assert layout[0] == 3 and layout[1] == 1
            a, n = struct.unpack_from("<QQ", layout, 2)
            assert a + n <= len(b)
            return "dataset"
        assert types[:2] == [2, 10]  # Link Info, Group Info
        tree = {}
        for t, m in msgs:
            if t != 6:
                continue
            assert m[0] == 1 and m[1] == 0
            name = m[3:3 + m[2]].decode()
            child = struct.unpack_from("<Q", m, 3 + m[2])[0]
            tree[name] = walk(child, depth + 1)
        return tree

    return walk(root)


def test_file_structure_independent_parse(engine, written):
    tree = _parse(engine, written)
    assert tree["Histogram"]["1"]["Histogram"] == "dataset"
    assert tree["Lattice"]["0"]["-8"]["Lattice"] == "dataset"
    assert tree["0"]["12345"]["Thu_Dec__3_18:00:00_2026"]["log_g"] == "dataset"


def test_corrupted_file_rejected(engine, written, tmp_path):
    b = bytearray(open(written, "rb").read())
    b[100] ^= 0xFF  # inside the root object header
    bad = tmp_path / "bad.h5"
    bad.write_bytes(bytes(b))
    with pytest.raises(engine.WlgError):
        engine.h5_list(str(bad))


def test_damaged_files_fail_cleanly(engine, written, tmp_path):
    """Damaged copies of a file in the engine's own structure (superblock 2,
    version-2 headers, checksums): every reader call returns a status; the
    child process neither crashes nor hangs."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import h5fuzz
    h5fuzz.check(engine.LIB, written, tmp_path)
