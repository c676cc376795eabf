"""GB300-native replica-exchange Wang-Landau engine (Python mirror of the C ABI).

The engine is ``libwlg.so`` (CUDA kernels for sm_103a + C++20 host code),
built in-tree by :func:`build`.  This module binds its ``extern "C"`` entry
points (``include/wlg.h``) with ctypes; it contains no computation of its own
and there is no fallback: if the library is missing or a call fails, an
exception is raised.

Device buffers are passed as integer device addresses (e.g. a CUDA tensor's
``data_ptr()``), streams as integer ``cudaStream_t`` handles (0 = default).
"""

from __future__ import annotations

import ctypes as C
import os

from .build import LIB, build  # noqa: F401

_lib = None

P = C.c_void_p
i8, i32, u32, i64, u64, f32, f64, sz = (C.c_int8, C.c_int, C.c_uint, C.c_longlong, C.c_uint64, C.c_float, C.c_double,
                                         C.c_size_t)

# name -> argument types (all return wlg_status = int unless listed in _RESTYPE)
SIGNATURES = {
    "wlg_status_string": [i32],
    "wlg_version": [],
    "wlg_init_interactions": [P, sz, i32, i32, f32, P],
    "wlg_apply_error_class": [P, i32, i32, i32, C.c_char, P],
    "wlg_init_lattice": [P, i32, i32, sz, i32, i32, P],
    "wlg_calc_energy": [i32, P, P, P, P, i32, i32, sz, i32, P],
    "wlg_wang_landau_pre_run": [P, P, P, P, P, P, P, P, i32, i32, i32, i32, i32, i32, u32, i32, sz, i32, i32, P],
    "wlg_wang_landau": [P] * 17 + [i32] * 8 + [P],
    "wlg_check_histogram": [P] * 9 + [f64, i32, i32, i32, P],
    "wlg_average_log_g": [P] * 8 + [i32, i32, i32, P],
    "wlg_reset_cond": [P, P, i32, f64, i32, P],
    "wlg_check_finished": [P, P, i32, i32, P],
    "wlg_replica_exchange": [P] * 9 + [i32] * 6 + [P],
    "wlg_max_int": [P, sz, P, P],
    "wlg_max_f64_nonneg": [P, sz, P, P],
    "wlg_uniforms": [u64, u64, u64, i32, P, P],
}
_RESTYPE = {"wlg_status_string": C.c_char_p, "wlg_version": C.c_char_p}


class WlgError(RuntimeError):
    def __init__(self, fn: str, status: int, text: str):
        super().__init__(f"{fn} failed: {text} (status {status})")
        self.status = status


def lib():
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise ImportError(f"{LIB} is missing: run qec_pf_wang_landau_gb300.build() first")
        L = C.CDLL(LIB)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, i32)
        _lib = L
    return _lib


def call(name: str, *args) -> None:
    """Call an entry point and raise WlgError on a non-OK status."""
    st = getattr(lib(), name)(*args)
    if st != 0:
        raise WlgError(name, st, lib().wlg_status_string(st).decode())


def version() -> str:
    return lib().wlg_version().decode()
