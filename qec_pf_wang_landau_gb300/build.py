"""Build recipe for the engine's shared library (``libwlg.so``) and the
prerun/mainrun programs (``bin/wlg_prerun``, ``bin/wlg_mainrun``).

Every ``csrc/*.cu`` translation unit is compiled by nvcc for sm_103a only,
every ``csrc/*.cpp`` host unit by g++, in parallel, and all are linked into
one in-tree shared library exposing the C ABI of ``include/wlg.h``; each
``cli/*.cpp`` becomes a program linked against it.  Host code is built with
``-ffp-contract=off`` so float expressions round identically on x86 and Arm.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libwlg.so")
CLI = os.path.join(PKG, "cli")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++20", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-std=c++20", "-O3", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + os.path.join(ROOT, "include")]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                  + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc))) if nvcc else "/usr/local/cuda"


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    if src.endswith(".cpp"):
        cmd = ["g++", *CXX_FLAGS, "-I" + os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj + ".tmp"]
    else:
        cmd = ["nvcc", *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    if force:
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        subprocess.run(["nvcc", *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart", "-lpthread"], check=True)
        os.replace(LIB + ".tmp", LIB)
    build_programs(force)
    return LIB


def build_programs(force: bool = False) -> list:
    """bin/wlg_<name> for every cli/<name>.cpp, linked against libwlg.so (rpath $ORIGIN/..)."""
    os.makedirs(BIN, exist_ok=True)
    deps = [LIB] + glob.glob(os.path.join(CLI, "*.h")) + _headers()
    out = []
    for src in sorted(glob.glob(os.path.join(CLI, "*.cpp"))):
        exe = os.path.join(BIN, "wlg_" + os.path.splitext(os.path.basename(src))[0])
        newest = max(os.path.getmtime(d) for d in deps + [src])
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < newest:
            subprocess.run(["g++", *CXX_FLAGS, "-I" + os.path.join(_cuda_home(), "include"), src, "-o", exe + ".tmp",
                            "-L" + PKG, "-lwlg", "-Wl,-rpath,$ORIGIN/.."], check=True)
            os.replace(exe + ".tmp", exe)
        out.append(exe)
    return out


if __name__ == "__main__":
    print(build())
