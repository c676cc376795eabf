"""CPU test of the engine's host worker pool (csrc/wlg_pool.h), which runs
the per-problem hand-off and stitching of a batch: every index exactly once
per job, exceptions reach the caller, the pool survives them."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_worker_pool(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "pool_check"
    subprocess.run([cxx, "-std=c++20", "-O2", "-pthread", "-I" + os.path.join(ROOT, "qec_pf_wang_landau_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "csrc", "pool_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
