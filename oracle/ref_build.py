"""Build recipe of the reference harness — test/benchmark infrastructure.

* build_cubin(): compiles the reference's unmodified kernel library
  (src/wl.cu of dfki-ric-quantum/qec_pf_wang_landau, read where it lies)
  into oracle/_ref/wl_ref.cubin for sm_103a.  Runs only where the reference
  sources exist; the cubin (device code, git-ignored) travels with the tree.
* build_harness(): compiles oracle/ref_harness.cu (this project's own driver
  of those kernels) into oracle/_ref/libref_harness.so.
* build_host(): compiles oracle/ref_host.cpp, which includes the reference's
  unmodified src/interval.cpp, src/result_handling.cpp and src/file_io.cpp
  (the latter against the test-only HDF5 declarations of oracle/h5stub) where
  they lie,
  into oracle/_ref/libref_host.so (host code; only where the reference
  sources exist, since the x86 library does not travel).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT, "wl_ref.cubin")
HARNESS = os.path.join(OUT, "libref_harness.so")
HOST = os.path.join(OUT, "libref_host.so")
# where the reference project's sources lie (only read when present)
REFERENCE = os.environ.get("WLG_REFERENCE_DIR", "/root/reference")


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


def build_host() -> str | None:
    srcs = [os.path.join(REFERENCE, "src", f) for f in ("interval.cpp", "result_handling.cpp", "file_io.cpp")]
    stub = os.path.join(HERE, "h5stub")
    drv = [os.path.join(HERE, "ref_host.cpp"), os.path.join(stub, "hdf5.h"), os.path.join(stub, "h5stub.inc")]
    if not all(os.path.exists(f) for f in srcs):
        return None
    os.makedirs(OUT, exist_ok=True)
    newest = max(os.path.getmtime(f) for f in srcs + drv)
    if os.path.exists(HOST) and os.path.getmtime(HOST) >= newest:
        return HOST
    # the test-only HDF5 declarations come first on the include path: file_io.cpp
    # is compiled for its in-memory hand-off functions only
    subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-Wl,-Bsymbolic-functions", "-I" + stub,
                    "-I" + os.path.join(REFERENCE, "src"), "-o", HOST + ".tmp", drv[0]], check=True)
    os.replace(HOST + ".tmp", HOST)
    return HOST


def build() -> tuple[str | None, str]:
    build_host()
    return build_cubin(), build_harness()
