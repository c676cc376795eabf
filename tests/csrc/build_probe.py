"""Builds the test-only cuRAND probe library (tests/csrc/libprobe.so)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libprobe.so")


def build() -> str:
    src = os.path.join(HERE, "curand_probe.cu")
    csrc = os.path.join(HERE, "..", "..", "qec_pf_wang_landau_gb300", "csrc")
    deps = [src] + [os.path.join(csrc, f) for f in ("wlg_shadow.cuh", "wlg_accept.cuh", "wlg_rng.cuh")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in deps):
        return LIB
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
                    "-shared", "-o", LIB + ".tmp", src], check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB
