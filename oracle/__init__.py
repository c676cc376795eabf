"""ORACLE — test infrastructure only.

ctypes binding to ``liboracle.so``, the CPU restatement of the reference's
replica-exchange Wang-Landau path (oracle.cpp, oracle_host.cpp).  Only the
test-suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
it, to compare the engine's results with; the engine never imports it.

``build()`` is the build recipe: one g++ invocation, no external libraries.
Host float arithmetic is compiled with ``-ffp-contract=off`` so that the
reference's float expressions (interval.cpp:17-20) round the same way on x86
and Arm hosts.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = ["oracle.cpp", "oracle_host.cpp"]

_lib = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdr = os.path.join(HERE, "oracle_core.h")
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in srcs + [hdr])
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB + ".tmp", *srcs,
           "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _declare(_lib)
    return _lib


P = C.c_void_p
i32, u32, i64, u64, f32, f64, sz = C.c_int, C.c_uint, C.c_longlong, C.c_uint64, C.c_float, C.c_double, C.c_size_t


def _declare(L):
    sig = {
        "orc_philox_raw": (None, [u64, u64, u64, i32, P]),
        "orc_uniform": (None, [u64, u64, u64, i32, P]),
        "orc_raw_to_uniform": (f32, [u32]),
        "orc_interval_results": (i32, [i32, i32, u32, i32, f32, P, P, P, P]),
        "orc_init_interactions": (None, [P, sz, i32, i32, f32]),
        "orc_apply_horizontal_error": (None, [P, i32, i32, i32]),
        "orc_apply_vertical_error": (None, [P, i32, i32, i32]),
        "orc_apply_error_class": (None, [P, i32, i32, i32, C.c_char]),
        "orc_init_lattice": (None, [P, i32, i32, sz, i32, i32]),
        "orc_calc_energy": (None, [i32, P, P, P, P, i32, i32, sz, i32]),
        "orc_wang_landau_pre_run": (None, [P, P, P, P, P, P, P, P, i32, i32, i32, i32, i32, i32, u32, i32, sz, i32,
                                           i32]),
        "orc_wang_landau": (i32, [P] * 17 + [i32] * 8),
        "orc_check_histogram": (None, [P] * 9 + [f64, i32, i32, i32]),
        "orc_average_log_g": (None, [P] * 8 + [i32, i32, i32]),
        "orc_reset_cond": (None, [P, P, i32, f64, i32]),
        "orc_check_finished": (None, [P, P, i32, i32]),
        "orc_replica_exchange": (None, [P] * 9 + [i32] * 6),
        "orc_prerun": (None, [i32, i32, i32, f32, C.c_char, i32, i32, i32, i32, i32, P, P, P, P, P]),
        "orc_mainrun": (i32, [i32, i32, i32, i32, i32, i32, f32, f64, f64, i32, i32, i32, i32, i32, i64] + [P] * 5
                        + [i32] + [P] * 8),
        "orc_stitch": (i32, [P, P, P, i32, i32, i32, i32, P, P, i32, P, i32]),
        "orc_exact_counts": (None, [P, i32, i32, i32, P]),
        "orc_enumerate_counts": (None, [P, i32, i32, i32, P]),
        "orc_log_partition": (f64, [P, P, i32, f64]),
        "orc_run_problems": (i64, [P, i32, i32, P, P, P]),
        "orc_exp_log": (None, [P, P, P, i32]),
        "orc_sqrt_chain": (None, [f64, i32, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


# ----------------------------------------------------------------- wrappers --

def uniforms(key: int, subseq: int, offset: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().orc_uniform(key, subseq, offset, n, ptr(out))
    return out


def philox_raw(key: int, subseq: int, offset: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_philox_raw(key, subseq, offset, n, ptr(out))
    return out


def interval_results(e_min, e_max, n_int, walkers, overlap):
    """interval.cpp:5-41 -> (start, end, len_hist_all, len_interval); raises ValueError like the reference."""
    s = np.zeros(n_int, np.int32)
    e = np.zeros(n_int, np.int32)
    tot = C.c_longlong(0)
    ln = C.c_int(0)
    rc = lib().orc_interval_results(e_min, e_max, n_int, walkers, C.c_float(overlap), ptr(s), ptr(e),
                                    C.byref(tot), C.byref(ln))
    if rc == 1:
        raise ValueError("Overlap is out of bounds.")
    if rc == 2:
        raise ValueError("The interval arguments create empty intervals.")
    return s, e, tot.value, ln.value


def init_interactions(X, Y, R, seed, prob, cls="i"):
    J = np.zeros(R * 2 * X * Y, np.int8)
    lib().orc_init_interactions(ptr(J), X * Y, R, seed, C.c_float(prob))
    lib().orc_apply_error_class(ptr(J), X, Y, R, cls.encode())
    return J


def init_lattice(X, Y, num_lattices, seed, wpi):
    lat = np.zeros(num_lattices * X * Y, np.int8)
    lib().orc_init_lattice(ptr(lat), X, Y, num_lattices, seed, wpi)
    return lat


def calc_energy(boundary, lat, J, off_lat, X, Y, num_lattices, wpi):
    E = np.zeros(num_lattices, np.int32)
    lib().orc_calc_energy(boundary, ptr(E), ptr(lat), ptr(J), ptr(off_lat), X, Y, num_lattices, wpi)
    return E


def exact_counts(J, X, Y, boundary, brute=False):
    c = np.zeros(4 * X * Y + 1, np.float64)
    fn = lib().orc_enumerate_counts if brute else lib().orc_exact_counts
    fn(ptr(np.ascontiguousarray(J, np.int8)), X, Y, boundary, ptr(c))
    return c


class OrcProblem(C.Structure):
    _fields_ = [("X", i32), ("Y", i32), ("boundary", i32), ("prob", f32), ("error_class", i32), ("seed", i32),
                ("sample", i32), ("pre_walkers", i32), ("pre_intervals", i32), ("pre_iterations", i32),
                ("n_int", i32), ("W", i32), ("overlap", f32), ("alpha", f64), ("beta", f64), ("n_iter", i32),
                ("exchange_every", i32), ("exchange_mode", i32), ("max_outer", i64)]


def run_problems(problems, threads):
    """Whole problems (pre-run + main run) on host threads; returns (status, outer, flips)."""
    n = len(problems)
    arr = (OrcProblem * n)(*problems)
    st = np.zeros(n, np.int32)
    outer = np.zeros(n, np.int64)
    fl = np.zeros(n, np.int64)
    lib().orc_run_problems(C.cast(arr, C.c_void_p), n, threads, ptr(st), ptr(outer), ptr(fl))
    return st, outer, fl


# ------------------------------------------------------ reference harness --

_ref = None


def reference_harness():
    """ctypes handle of oracle/_ref/libref_harness.so with the reference's
    cubin loaded, or None when the cubin is not available."""
    global _ref
    if _ref is None:
        from . import ref_build
        cubin, so = ref_build.build()
        if cubin is None or not os.path.exists(cubin):
            return None
        L = C.CDLL(so)
        L.refh_open.argtypes = [C.c_char_p]
        L.refh_open.restype = C.c_int
        L.refh_run.argtypes = [i32, i32, i32, f32, C.c_char, i32, i32, i32, i32, i32, i32, i32, f32, f64, f64, i32, i32,
                               i64, P, P, P, P, P, P, i64]
        L.refh_run.restype = C.c_int
        L.refh_mainrun.argtypes = [i32, i32, i32, i32, i32, i32, P, P, P, P, i32, i32, f32, f64, f64, i32, i32, i64,
                                   P, P, P, P, P, i64]
        L.refh_mainrun.restype = C.c_int
        kernels = {
            "refh_k_init_interactions": [P, i32, i32, i32, i32, f32, C.c_char],
            "refh_k_calc_energy": [i32, P, P, P, P, i32, i32, sz, i32],
            "refh_k_pre_run": [P] * 8 + [i32] * 6 + [u32, i32, sz, i32, i32],
            "refh_k_init_offsets_histogram": [P] * 4 + [i32] * 3,
            "refh_k_wang_landau": [P] * 17 + [i32] * 8,
            "refh_k_check_histogram": [P] * 9 + [f64, i32, i32, i32],
            "refh_k_average_log_g": [P] * 8 + [i32] * 3,
            "refh_k_reset_cond": [P, P, i32, f64, i32, i32, i32],
            "refh_k_check_finished": [P, P, i32, i32],
            "refh_k_replica_exchange": [P] * 9 + [i32] * 5,
        }
        for name, args in kernels.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        rc = L.refh_open(cubin.encode())
        if rc != 0:
            raise RuntimeError(f"reference cubin could not be loaded (code {rc})")
        _ref = L
    return _ref


_ref_host = None


def reference_host():
    """ctypes handle of oracle/_ref/libref_host.so (the reference's own
    interval.cpp and result_handling.cpp), or None where the reference
    sources are absent."""
    global _ref_host
    if _ref_host is None:
        from . import ref_build
        so = ref_build.build_host()
        if so is None:
            return None
        L = C.CDLL(so)
        L.ref_interval.argtypes = [i32, i32, C.c_uint, i32, f32, P, P, P, P]
        L.ref_interval.restype = C.c_int
        L.ref_stitch.argtypes = [P, i64, P, P, i32, i32, i32, i32, P, P, i32, P]
        L.ref_stitch.restype = C.c_int
        L.ref_handoff.argtypes = [i32] * 6 + [f32] + [P] * 12 + [i64]
        L.ref_handoff.restype = C.c_int
        _ref_host = L
    return _ref_host


def ref_interval(e_min, e_max, n_int, walkers, overlap):
    """interval.cpp of the reference: (starts, ends, total, len) or None when it throws."""
    L = reference_host()
    s = np.zeros(n_int, np.int32)
    e = np.zeros(n_int, np.int32)
    tot, ln = C.c_longlong(0), C.c_int(0)
    if L.ref_interval(e_min, e_max, n_int, walkers, C.c_float(overlap), ptr(s), ptr(e), C.byref(tot), C.byref(ln)):
        return None
    return s, e, tot.value, ln.value


def ref_stitch(logG, start, end, n_int, W, X, Y):
    """result_handling.cpp of the reference: (rc, E, log g) it would write."""
    L = reference_host()
    cap = 4 * X * Y + 1 + 4 * n_int
    E = np.zeros(cap, np.int32)
    G = np.zeros(cap, np.float64)
    n = C.c_int(0)
    lg = np.ascontiguousarray(logG, np.float64)
    s, e = np.ascontiguousarray(start, np.int32), np.ascontiguousarray(end, np.int32)
    rc = L.ref_stitch(ptr(lg), len(lg), ptr(s), ptr(e), n_int, W, X, Y, ptr(E), ptr(G), cap, C.byref(n))
    return rc, E[:n.value].copy(), G[:n.value].copy()


def stitch(logG, start, end, n_int, W, X, Y, mode=0):
    """The oracle's restatement of result_handling.cpp: (rc, E, log g).
    mode 0: the reference's phantom successor at a window's last key; 1: skipped."""
    cap = 4 * X * Y + 1 + 4 * n_int
    E = np.zeros(cap, np.int32)
    G = np.zeros(cap, np.float64)
    n = C.c_int(0)
    lg = np.ascontiguousarray(logG, np.float64)
    s, e = np.ascontiguousarray(start, np.int32), np.ascontiguousarray(end, np.int32)
    rc = lib().orc_stitch(ptr(lg), ptr(s), ptr(e), n_int, W, X, Y, ptr(E), ptr(G), cap, C.byref(n), mode)
    return rc, E[:n.value].copy(), G[:n.value].copy()


def reference_run(X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n, I, W, overlap, alpha, beta, n_iter, xc,
                  max_outer=0, want_raw=True):
    """The reference's own kernels, prerun.cu then mainrun.cu order, for R samples.
    Returns dict(status, pre_ms, main_ms, outer, start, end, windows)."""
    L = reference_harness()
    if L is None:
        raise RuntimeError("reference cubin not available")
    t_pre, t_main, outer = C.c_double(), C.c_double(), C.c_longlong()
    starts = np.zeros(R * I, np.int32)
    ends = np.zeros(R * I, np.int32)
    cap = R * I * (4 * X * Y + 1)
    raw = np.zeros(cap if want_raw else 1, np.float64)
    st = L.refh_run(X, Y, boundary, C.c_float(prob), cls.encode(), seed, R, pre_w, pre_i, pre_n, I, W,
                    C.c_float(overlap), alpha, beta, n_iter, xc, max_outer, C.byref(t_pre), C.byref(t_main),
                    C.byref(outer), ptr(starts), ptr(ends), ptr(raw) if want_raw else None, cap)
    wins = []
    if want_raw and st == 0:
        pos = 0
        for q in range(R * I):
            ln = int(ends[q] - starts[q] + 1)
            wins.append(raw[pos:pos + ln].copy())
            pos += ln
    return dict(status=st, pre_ms=t_pre.value, main_ms=t_main.value, outer=outer.value, start=starts, end=ends,
                windows=wins)


def reference_mainrun(X, Y, boundary, seed, R, pre_i, seen, couplings, lattices, lattice_energy, I, W, overlap,
                      alpha, beta, n_iter, xc, max_outer=0):
    """mainrun.cu alone on the reference's own kernels, from pre-run outputs of
    samples 0..R-1 (seen [R][4N+1], couplings [R][2N], lattices [R][pre_i][N],
    zero where none was stored, lattice_energy [R][pre_i]).
    Returns dict(status, main_ms, outer, start, end, windows)."""
    L = reference_harness()
    if L is None:
        raise RuntimeError("reference cubin not available")
    t_main, outer = C.c_double(), C.c_longlong()
    starts = np.zeros(R * I, np.int32)
    ends = np.zeros(R * I, np.int32)
    cap = R * I * (4 * X * Y + 1)
    raw = np.zeros(cap, np.float64)
    a = [np.ascontiguousarray(seen, np.uint8), np.ascontiguousarray(couplings, np.int8),
         np.ascontiguousarray(lattices, np.int8), np.ascontiguousarray(lattice_energy, np.int32)]
    st = L.refh_mainrun(X, Y, boundary, seed, R, pre_i, ptr(a[0]), ptr(a[1]), ptr(a[2]), ptr(a[3]), I, W,
                        C.c_float(overlap), alpha, beta, n_iter, xc, max_outer, C.byref(t_main), C.byref(outer),
                        ptr(starts), ptr(ends), ptr(raw), cap)
    wins = []
    if st in (0, 3):
        pos = 0
        for q in range(R * I):
            ln = int(ends[q] - starts[q] + 1)
            wins.append(raw[pos:pos + ln].copy())
            pos += ln
    return dict(status=st, main_ms=t_main.value, outer=outer.value, start=starts, end=ends, windows=wins)


def ref_handoff(X, Y, R, pre_i, I, W, overlap, seen, found, found_energy, lattices):
    """The reference's own hand-off (file_io.cpp:558-659 with interval.cpp, as
    mainrun.cu chains them) on pre-run outputs of samples 0..R-1.  Returns None
    when it throws, else dict(spectrum, off_spec, len_spec, e_min, e_max,
    start, end, lattices [R*I*W][N])."""
    L = reference_host()
    N = X * Y
    spec = np.zeros(R * (4 * N + 1), np.int8)
    off = np.zeros(R, np.int32)
    ln = np.zeros(R, np.int32)
    lo = np.zeros(R, np.int32)
    hi = np.zeros(R, np.int32)
    s = np.zeros(R * I, np.int32)
    e = np.zeros(R * I, np.int32)
    lat = np.zeros(R * I * W * N, np.int8)
    ins = [np.ascontiguousarray(seen, np.uint8), np.ascontiguousarray(found, np.int32),
           np.ascontiguousarray(found_energy, np.int32), np.ascontiguousarray(lattices, np.int8)]
    rc = L.ref_handoff(X, Y, R, pre_i, I, W, C.c_float(overlap), *(ptr(a) for a in ins), ptr(spec), ptr(off), ptr(ln),
                       ptr(lo), ptr(hi), ptr(s), ptr(e), ptr(lat), len(spec))
    if rc != 0:
        return None
    return dict(spectrum=spec[:int(ln.sum())], off_spec=off, len_spec=ln, e_min=lo, e_max=hi, start=s, end=e,
                lattices=lat.reshape(R * I * W, N))
