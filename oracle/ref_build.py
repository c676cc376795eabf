"""Build recipe of the reference harness — test/benchmark infrastructure.

* build_cubin(): compiles the reference's unmodified kernel library
  (src/wl.cu of dfki-ric-quantum/qec_pf_wang_landau, read where it lies)
  into oracle/_ref/wl_ref.cubin for sm_103a.  Runs only where the reference
  sources exist; the cubin (device code, git-ignored) travels with the tree.
* build_harness(): compiles oracle/ref_harness.cu (this project's own driver
  of those kernels) into oracle/_ref/libref_harness.so.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT, "wl_ref.cubin")
HARNESS = os.path.join(OUT, "libref_harness.so")
REFERENCE = "/root/reference"


def build_cubin() -> str | None:
    src = os.path.join(REFERENCE, "src", "wl.cu")
    if not os.path.exists(src):
        return CUBIN if os.path.exists(CUBIN) else None
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(src):
        return CUBIN
    subprocess.run(["nvcc", "-std=c++20", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + os.path.join(REFERENCE, "src"), "-o", CUBIN + ".tmp", src], check=True)
    os.replace(CUBIN + ".tmp", CUBIN)
    return CUBIN


def build_harness() -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cu")
    if os.path.exists(HARNESS) and os.path.getmtime(HARNESS) >= os.path.getmtime(src):
        return HARNESS
    subprocess.run(["nvcc", "-std=c++20", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
                    "-shared", "-o", HARNESS + ".tmp", src, "-lcuda"], check=True)
    os.replace(HARNESS + ".tmp", HARNESS)
    return HARNESS


def build() -> tuple[str | None, str]:
    return build_cubin(), build_harness()
