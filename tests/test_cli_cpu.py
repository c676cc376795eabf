"""The command-line programs on CPU: what they decide before any device
work (options, help, pre-run file checks).  No GPU is needed: each case
exits before the engine is created."""
import os
import subprocess
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import h5v0  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "qec_pf_wang_landau_gb300", "bin")
MAIN = ["-x", "4", "-y", "4", "-n", "1000", "-p", "0.04", "-a", "0.8", "-b", "0.001", "-i", "10", "-w", "3",
        "-o", "0.25", "-s", "12345", "-e", "i", "-r", "2", "-c", "20", "-d", "7", "-f", "3600"]
SUB = "task_id_7/seed_12345/periodic/prob_0.040000/X_4_Y_4/error_class_i"


@pytest.fixture(scope="module")
def built():
    import qec_pf_wang_landau_gb300 as wlg
    wlg.build()
    return wlg


def run(prog, args, cwd):
    return subprocess.run([os.path.join(BIN, prog), *args], cwd=cwd, capture_output=True, text=True, timeout=120)


def prerun_file(tmp_path, interaction=None, lattice=None):
    N = 16
    tree = {"Histogram": {}, "Interaction": {}, "Lattice": {}}
    for k in range(2):
        tree["Histogram"][str(k)] = {"Histogram": h5v0.Dataset(np.ones(4 * N + 1, np.uint64))}
        J = np.ones(2 * N, np.int8) if interaction is None else interaction
        tree["Interaction"][str(k)] = {"Interaction": h5v0.Dataset(J)}
        lat = -np.ones(N, np.int8) if lattice is None else lattice
        tree["Lattice"][str(k)] = {"-32": {"Lattice": h5v0.Dataset(lat)}}
    d = tmp_path / "init" / SUB
    d.mkdir(parents=True)
    h5v0.write(str(d / "prerun_results.h5"), tree)


def test_help_version_and_missing_options(built, tmp_path):
    for prog in ("wlg_prerun", "wlg_mainrun", "wlg_decode"):
        assert run(prog, ["--help"], tmp_path).returncode == 0
        assert "version" in run(prog, ["-v"], tmp_path).stdout
    r = run("wlg_decode", ["-x", "4"], tmp_path)
    assert r.returncode != 0 and "required" in r.stderr


def test_mainrun_without_a_prerun_file_fails(built, tmp_path):
    r = run("wlg_mainrun", MAIN, tmp_path)
    assert r.returncode != 0 and "Could not open HDF5 file" in r.stderr


@pytest.mark.parametrize("what", ["interaction", "lattice"])
def test_mainrun_refuses_values_other_than_pm1(built, tmp_path, what):
    bad = np.ones(32 if what == "interaction" else 16, np.int8)
    bad[3] = 0
    prerun_file(tmp_path, **{what: bad})
    r = run("wlg_mainrun", MAIN, tmp_path)
    assert r.returncode != 0 and "other than +-1" in r.stderr


def test_mainrun_refuses_wrong_histogram_length(built, tmp_path):
    N = 16
    tree = {"Histogram": {"0": {"Histogram": h5v0.Dataset(np.ones(4 * N, np.uint64))}},
            "Interaction": {"0": {"Interaction": h5v0.Dataset(np.ones(2 * N, np.int8))}}}
    d = tmp_path / "init" / SUB
    d.mkdir(parents=True)
    h5v0.write(str(d / "prerun_results.h5"), tree)
    r = run("wlg_mainrun", MAIN, tmp_path)
    assert r.returncode != 0 and "Histogram length" in r.stderr
