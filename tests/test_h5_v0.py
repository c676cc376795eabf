"""CPU tests: the engine's HDF5 reader on files in libhdf5's default
structure (superblock 0, version-1 object headers, symbol-table groups),
written by tests/h5v0.py from the public file-format specification — the
structure the reference's own prerun and mainrun produce.  No libhdf5 is
available here, so these files stand in for the reference's output."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import h5fuzz  # noqa: E402
import h5v0  # noqa: E402

KV = np.dtype({"names": ["Key", "Value"], "formats": ["<i4", "<f8"], "offsets": [0, 8], "itemsize": 16})


@pytest.fixture(scope="module")
def wlg():
    import qec_pf_wang_landau_gb300 as m
    m.build()
    return m


def prerun_like(R=3, N=16, energies=(-32, -24, -16, -8, 0, 8, 16, 24, 28, 30)):
    rng = np.random.default_rng(1)
    tree = {"Histogram": {}, "Interaction": {}, "Lattice": {}}
    for k in range(R):
        tree["Histogram"][str(k)] = {"Histogram": h5v0.Dataset((rng.random(4 * N + 1) < 0.5).astype(np.uint64))}
        tree["Interaction"][str(k)] = {"Interaction": h5v0.Dataset(np.where(rng.random(2 * N) < 0.1, -1, 1)
                                                                  .astype(np.int8))}
        tree["Lattice"][str(k)] = {str(e): {"Lattice": h5v0.Dataset(np.where(rng.random(N) < 0.5, -1, 1)
                                                                    .astype(np.int8))} for e in energies}
    return tree


def check_tree(wlg, path, tree, prefix=""):
    groups, datasets = wlg.h5_list(path, prefix)
    want_g = sorted(k for k, v in tree.items() if isinstance(v, dict) and not k.startswith("__"))
    want_d = sorted(k for k, v in tree.items() if isinstance(v, h5v0.Dataset))
    assert sorted(groups) == want_g and sorted(datasets) == want_d, prefix
    for k in want_d:
        ds = tree[k]
        got = wlg.h5_read(path, f"{prefix}/{k}")
        assert np.array_equal(got.view(np.uint8), np.ascontiguousarray(ds.data).view(np.uint8)), f"{prefix}/{k}"
        for name, value in ds.attrs.items():
            assert wlg.h5_attribute(path, f"{prefix}/{k}", name) == value
    for k in want_g:
        check_tree(wlg, path, tree[k], f"{prefix}/{k}")


def test_prerun_layout(wlg, tmp_path):
    tree = prerun_like()
    p = str(tmp_path / "prerun_results.h5")
    h5v0.write(p, tree)
    check_tree(wlg, p, tree)


def test_mainrun_layout_with_attribute_compact_and_continuation(wlg, tmp_path):
    kv = np.zeros(7, KV)
    kv["Key"] = np.arange(-12, 16, 4)
    kv["Value"] = np.linspace(0.5, 9.25, 7)
    tree = {str(k): {"12345": {"Mon_Jan__1_00:00:00_2024": {
        "log_g": h5v0.Dataset(kv, attrs={"CodeVersion": "v1.2-abc"}, continuation=(k == 1))}}} for k in range(3)}
    tree["2"]["12345"]["Mon_Jan__1_00:00:00_2024"]["small"] = h5v0.Dataset(np.arange(5, dtype=np.int32),
                                                                           compact=True)
    p = str(tmp_path / "mainrun_results.h5")
    h5v0.write(p, tree)
    check_tree(wlg, p, tree)


def test_large_groups_span_nodes_and_levels(wlg, tmp_path):
    """40 children: 5 symbol table nodes, and a two-level B-tree."""
    flat = {f"{e}": {"Lattice": h5v0.Dataset(np.full(9, e % 3 - 1, np.int8))} for e in range(-80, 80, 4)}
    tree = {"one_level": dict(flat), "two_levels": dict(flat, __two_levels__=True), "empty": {}}
    p = str(tmp_path / "big.h5")
    h5v0.write(p, tree)
    check_tree(wlg, p, tree)


def test_unsupported_structures_fail_cleanly(wlg, tmp_path):
    p = str(tmp_path / "bad.h5")
    h5v0.write(p, {"a": {"x": h5v0.Dataset(np.zeros(3, np.int16))}})  # int16: not a type the reference writes
    with pytest.raises(wlg.WlgError):
        wlg.h5_read(p, "/a/x")
    with open(p, "r+b") as f:  # superblock version 4 does not exist
        f.seek(8)
        f.write(b"\x04")
    with pytest.raises(wlg.WlgError):
        wlg.h5_list(p, "")


def test_link_back_to_an_enclosing_group_is_refused(wlg, tmp_path):
    """A symbol-table entry pointing back at the root group (a cycle) ends
    the parse with an error instead of recursing."""
    import struct
    p = str(tmp_path / "cycle.h5")
    h5v0.write(p, {"a": {"b": h5v0.Dataset(np.zeros(3, np.int8))}})
    b = bytearray(open(p, "rb").read())
    root = struct.unpack_from("<Q", b, 64)[0]  # superblock 0: root entry's object header address
    snod = b.index(b"SNOD")  # group a's node (children are written before their parents)
    struct.pack_into("<Q", b, snod + 16, root)  # entry 0 ("b"): object header address
    open(p, "wb").write(bytes(b))
    with pytest.raises(wlg.WlgError):
        wlg.h5_list(p, "")


def test_damaged_files_fail_cleanly(wlg, tmp_path):
    """Randomly damaged files (bytes changed, truncations, addresses and
    lengths overwritten with extreme or in-file values) walked through every
    reader entry point in a child process: each call returns a status; the
    process neither crashes nor hangs."""
    src = str(tmp_path / "pre.h5")
    tree = prerun_like(R=2)
    tree["7"] = {"12345": {"Mon": {"log_g": h5v0.Dataset(np.zeros(5, KV), attrs={"CodeVersion": "x"},
                                                         continuation=True)}}}
    h5v0.write(src, tree)
    h5fuzz.check(wlg.LIB, src, tmp_path)
