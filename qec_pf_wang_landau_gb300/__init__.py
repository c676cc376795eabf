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
    "wlg_context_create": [i32, sz, P],
    "wlg_context_destroy": [P],
    "wlg_context_last_error": [P],
    "wlg_context_set_stream": [P, P],
    "wlg_context_set_stitching": [P, i32],
    "wlg_solve": [P, P, i32, P, P, P, i64],
    "wlg_solve_couplings": [P, P, i32, P, P, P, P, i64],
    "wlg_frustration": [i32, i32, i32, P, P],
    "wlg_couplings_from_syndrome": [i32, i32, i32, P, P],
    "wlg_solve_raw": [P, P, i32, P, P, P, P, i64, P],
    "wlg_last_stats": [P, P],
    "wlg_last_main_times": [P, P, P, i32, P],
    "wlg_handoff": [P, i32] + [P] * 12,
    "wlg_measure_peaks": [i32, P],
    "wlg_solve_plain": [P, i32, P, P, P, i64, P, P],
    "wlg_solve_raw_noalloc": [P, i32, P, P, P, P, i64, P, P],
    "wlg_class_log_probs": [P, P, P, P, i32, f64, P, P],
    "wlg_prerun": [P, P, i32, P, P, P, P, P],
    "wlg_mainrun": [P, P, i32, P, P, P, P, P, f64, P, P, P, i64],
    "wlg_h5_lookup3": [P, sz, u32],
    "wlg_h5_list": [C.c_char_p, C.c_char_p, P, sz],
    "wlg_h5_read": [C.c_char_p, C.c_char_p, P, P, P, u64],
    "wlg_h5_attribute": [C.c_char_p, C.c_char_p, C.c_char_p, P, sz],
    "wlg_context_autotune": [P, P, i32, i32, P, i32, P],
    "wlg_server_create": [i32, P, P],
    "wlg_server_submit": [P, P, i32, P],
    "wlg_server_submit_couplings": [P, P, i32, P, P],
    "wlg_server_poll": [P, P, i32, P, i32],
    "wlg_server_stats_get": [P, P],
    "wlg_server_destroy": [P],
    "wlg_server_last_error": [P],
}
_RESTYPE = {"wlg_status_string": C.c_char_p, "wlg_version": C.c_char_p, "wlg_context_last_error": C.c_char_p,
            "wlg_h5_lookup3": u32,
            "wlg_server_last_error": C.c_char_p}


def _couplings(problems, couplings):
    """Concatenated int8 bond patterns (None stays None)."""
    if couplings is None:
        return None
    import numpy as np
    parts = [np.ascontiguousarray(c, dtype=np.int8).ravel() for c in couplings]
    if len(parts) != len(problems) or any(len(c) != 2 * p.X * p.Y for c, p in zip(parts, problems)):
        raise ValueError("one bond pattern of 2*X*Y entries per problem")
    return np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros(1, np.int8))


def plaquettes(X: int, Y: int, boundary: int) -> int:
    """Number of plaquettes of an X x Y lattice (X*Y periodic, (X-1)*(Y-1) open)."""
    return X * Y if boundary == 0 else (X - 1) * (Y - 1)


def frustration(X: int, Y: int, boundary: int, couplings):
    """Syndrome (uint8 per plaquette, row-major) of a +-1 bond pattern (wlg_frustration)."""
    import numpy as np
    J = np.ascontiguousarray(couplings, dtype=np.int8).ravel()
    if len(J) != 2 * X * Y:
        raise ValueError("bond pattern needs 2*X*Y entries")
    out = np.zeros(max(plaquettes(X, Y, boundary), 1), np.uint8)
    call("wlg_frustration", X, Y, boundary, J.ctypes.data_as(P), out.ctypes.data_as(P))
    return out[:plaquettes(X, Y, boundary)]


def couplings_from_syndrome(X: int, Y: int, boundary: int, syndrome):
    """A +-1 bond pattern whose frustrated plaquettes are the syndrome (wlg_couplings_from_syndrome)."""
    import numpy as np
    S = np.ascontiguousarray(syndrome, dtype=np.uint8).ravel()
    if len(S) != plaquettes(X, Y, boundary):
        raise ValueError("syndrome needs one entry per plaquette")
    J = np.zeros(2 * X * Y, np.int8)
    call("wlg_couplings_from_syndrome", X, Y, boundary, S.ctypes.data_as(P), J.ctypes.data_as(P))
    return J


STITCH_REFERENCE, STITCH_DEFINED = 0, 1


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


# ------------------------------------------------------------------ engine --

WLG_OK, WLG_ERR_NEW_ENERGY, WLG_ERR_TIMEOUT, WLG_ERR_NO_LATTICE = 0, 3, 7, 5


class Problem(C.Structure):
    """wlg_problem: one disorder sample of one error class (see include/wlg.h)."""
    _fields_ = [("X", i32), ("Y", i32), ("boundary", i32), ("prob", f32), ("error_class", C.c_char), ("seed", i32),
                ("sample", i32), ("pre_walkers", i32), ("pre_intervals", i32), ("pre_iterations", i32),
                ("intervals", i32), ("walkers_per_interval", i32), ("overlap", f32), ("alpha", f64), ("beta", f64),
                ("iterations", i32), ("exchange_every", i32), ("exchange_mode", i32), ("global_parity", i32),
                ("max_outer", i64)]


class Result(C.Structure):
    _fields_ = [("status", i32), ("new_energy", i32), ("outer_iterations", i64), ("flips", i64), ("pre_flips", i64),
                ("n_energies", i32), ("offset", i64)]


def problem(X, Y, *, boundary=0, prob=0.04, error_class="i", seed=12345, sample=0, pre_walkers=128,
            pre_intervals=32, pre_iterations=1000, intervals=10, walkers_per_interval=3, overlap=0.25, alpha=0.8,
            beta=0.001, iterations=1000, exchange_every=20, exchange_mode=1, global_parity=0, max_outer=0):
    """A Problem with the reference's README defaults for the flags not given."""
    return Problem(X, Y, boundary, prob, error_class.encode() if isinstance(error_class, str) else error_class, seed,
                   sample, pre_walkers, pre_intervals, pre_iterations, intervals, walkers_per_interval, overlap,
                   alpha, beta, iterations, exchange_every, exchange_mode, global_parity, max_outer)


class Context:
    """An engine context on one CUDA device (owns its stream and device buffers)."""

    def __init__(self, device: int = 0, mem_budget_bytes: int = 0):
        h = C.c_void_p()
        call("wlg_context_create", device, mem_budget_bytes, C.byref(h))
        self._h = h

    def close(self):
        if self._h:
            lib().wlg_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, name, st):
        if st != 0:
            detail = lib().wlg_context_last_error(self._h).decode()
            raise WlgError(name, st, f"{lib().wlg_status_string(st).decode()}: {detail}")

    def solve(self, problems, couplings=None):
        """Stitched, normalised log g per problem: list of (Result, energies, log_g) (numpy arrays).
        couplings: None (drawn from seed and sample) or one class-'i' bond pattern (+-1, 2*X*Y) per
        problem (wlg_solve_couplings)."""
        import numpy as np
        n = len(problems)
        arr = (Problem * n)(*problems)
        res = (Result * n)()
        cap = sum(4 * p.X * p.Y + 1 for p in problems)
        E = np.zeros(max(cap, 1), np.int32)
        G = np.zeros(max(cap, 1), np.float64)
        J = _couplings(problems, couplings)
        self._check("wlg_solve_couplings",
                    lib().wlg_solve_couplings(self._h, C.cast(arr, P), n, None if J is None else J.ctypes.data_as(P),
                                              C.cast(res, P), E.ctypes.data_as(P), G.ctypes.data_as(P), cap))
        out = []
        for r in res:
            a, b = r.offset, r.offset + r.n_energies
            out.append((r, E[a:b].copy(), G[a:b].copy()))
        return out

    def solve_raw(self, problems):
        """Walker-0 log g of every window (dense, reference layout) per problem:
        list of (Result, starts, ends, [window arrays])."""
        import numpy as np
        n = len(problems)
        arr = (Problem * n)(*problems)
        res = (Result * n)()
        n_win = sum(p.intervals for p in problems)
        ws = np.zeros(max(n_win, 1), np.int32)
        we = np.zeros(max(n_win, 1), np.int32)
        cap = sum(p.intervals * (4 * p.X * p.Y + 1) for p in problems)
        raw = np.zeros(max(cap, 1), np.float64)
        off = np.zeros(max(n, 1), np.int64)
        self._check("wlg_solve_raw", lib().wlg_solve_raw(self._h, C.cast(arr, P), n, C.cast(res, P),
                                                          ws.ctypes.data_as(P), we.ctypes.data_as(P),
                                                          raw.ctypes.data_as(P), cap, off.ctypes.data_as(P)))
        out, wpos = [], 0
        for p, q in enumerate(problems):
            s = ws[wpos:wpos + q.intervals].copy()
            e = we[wpos:wpos + q.intervals].copy()
            wpos += q.intervals
            wins, pos = [], int(off[p])
            if res[p].status in (WLG_OK, WLG_ERR_TIMEOUT):
                for b in range(q.intervals):
                    ln = int(e[b] - s[b] + 1)
                    wins.append(raw[pos:pos + ln].copy())
                    pos += ln
            out.append((res[p], s, e, wins))
        return out

    def set_stream(self, stream=None):
        """Run later solves on a CUDA stream handle (int, e.g. torch's
        Stream.cuda_stream); None: the context's own stream."""
        self._check("wlg_context_set_stream",
                    lib().wlg_context_set_stream(self._h, C.c_void_p(stream) if stream else None))

    def set_stitching(self, mode: int):
        """STITCH_REFERENCE (default: the reference's output bins) or STITCH_DEFINED for later solves."""
        self._check("wlg_context_set_stitching", lib().wlg_context_set_stitching(self._h, mode))

    def autotune(self, problems, max_outer: int = 2):
        """Time teams-per-CTA choices on `problems` (capped at max_outer outer
        iterations) and keep the fastest per (form, team size) for later solves."""
        n = len(problems)
        arr = (Problem * n)(*problems)
        out = (Tuning * 16)()
        k = i32(0)
        self._check("wlg_context_autotune", lib().wlg_context_autotune(self._h, C.cast(arr, P), n, max_outer,
                                                                        C.cast(out, P), 16, C.byref(k)))
        return [{f: getattr(out[i], f) for f, _ in Tuning._fields_} for i in range(min(k.value, 16))]

    def stats(self):
        """What the last solve did: ms by phase, bytes copied each way, kernels launched."""
        st = Stats()
        call("wlg_last_stats", self._h, C.byref(st))
        return {f: getattr(st, f) for f, _ in Stats._fields_}

    def main_times(self):
        """Per problem of the last solve: (start_ms, end_ms) of its main run by
        the device clock, from the first start; -1 where none ran."""
        import numpy as np
        k = i32(0)
        lib().wlg_last_main_times(self._h, None, None, 0, C.byref(k))
        a = np.zeros(max(k.value, 1))
        b = np.zeros(max(k.value, 1))
        call("wlg_last_main_times", self._h, a.ctypes.data_as(P), b.ctypes.data_as(P), k.value, C.byref(k))
        return a[:k.value], b[:k.value]


class Tuning(C.Structure):
    _fields_ = [("form", i32), ("team", i32), ("per_cta", i32), ("main_ms", f32), ("candidates", i32)]


class Stats(C.Structure):
    _fields_ = [("pre_ms", f64), ("handoff_ms", f64), ("main_ms", f64), ("stitch_ms", f64), ("h2d_bytes", i64),
                ("d2h_bytes", i64), ("kernel_launches", i32), ("main_forms", i32)]


class Peaks(C.Structure):
    _fields_ = [("sm_count", i32), ("smem_gbs", f64), ("philox_draws_per_s", f64), ("exp_f64_per_s", f64),
                ("log_f64_per_s", f64)]


def measure_peaks(device: int = 0):
    """Secondary ceilings of the WL step measured on the device (wlg_measure_peaks)."""
    pk = Peaks()
    call("wlg_measure_peaks", device, C.byref(pk))
    return {f: getattr(pk, f) for f, _ in Peaks._fields_}


def handoff(problems, seen, couplings, found, found_energy, lattices):
    """wlg_handoff: the pre-run -> main-run hand-off on the host, from pre-run
    outputs in wlg_prerun's layout.  Per problem: dict(status, e_min, e_max,
    spectrum [4N+1], start [I], end [I], lattices [I][N])."""
    import numpy as np
    n = len(problems)
    arr = (Problem * n)(*problems)
    I = [p.intervals for p in problems]
    N = [p.X * p.Y for p in problems]
    st = np.zeros(n, np.int32)
    lo = np.zeros(n, np.int32)
    hi = np.zeros(n, np.int32)
    spec = np.zeros(max(sum(4 * x + 1 for x in N), 1), np.uint8)
    ws = np.zeros(max(sum(I), 1), np.int32)
    we = np.zeros(max(sum(I), 1), np.int32)
    lat = np.zeros(max(sum(i * x for i, x in zip(I, N)), 1), np.int8)
    ins = [np.ascontiguousarray(seen, np.uint8), np.ascontiguousarray(couplings, np.int8),
           np.ascontiguousarray(found, np.int32), np.ascontiguousarray(found_energy, np.int32),
           np.ascontiguousarray(lattices, np.int8)]
    call("wlg_handoff", C.cast(arr, P), n, *(a.ctypes.data_as(P) for a in ins), st.ctypes.data_as(P),
         lo.ctypes.data_as(P), hi.ctypes.data_as(P), spec.ctypes.data_as(P), ws.ctypes.data_as(P),
         we.ctypes.data_as(P), lat.ctypes.data_as(P))
    out, os_, ow, ol = [], 0, 0, 0
    for p in range(n):
        out.append(dict(status=int(st[p]), e_min=int(lo[p]), e_max=int(hi[p]), spectrum=spec[os_:os_ + 4 * N[p] + 1],
                        start=ws[ow:ow + I[p]], end=we[ow:ow + I[p]],
                        lattices=lat[ol:ol + I[p] * N[p]].reshape(I[p], N[p])))
        os_, ow, ol = os_ + 4 * N[p] + 1, ow + I[p], ol + I[p] * N[p]
    return out


def solve_plain(problems, stream=None):
    """The plain (reference-structured) form: list of (Result, energies, log_g), kernel launch count."""
    import numpy as np
    n = len(problems)
    arr = (Problem * n)(*problems)
    res = (Result * n)()
    cap = sum(4 * p.X * p.Y + 1 for p in problems)
    E = np.zeros(max(cap, 1), np.int32)
    G = np.zeros(max(cap, 1), np.float64)
    launches = C.c_longlong(0)
    call("wlg_solve_plain", C.cast(arr, P), n, C.cast(res, P), E.ctypes.data_as(P), G.ctypes.data_as(P), cap,
         stream, C.byref(launches))
    return [(r, E[r.offset:r.offset + r.n_energies].copy(), G[r.offset:r.offset + r.n_energies].copy())
            for r in res], launches.value


def class_log_probs(curves, prob):
    """Nishimori-temperature log-probabilities of logical classes from their
    normalised (energies, log_g) curves; returns (log_z, log_probs)."""
    import numpy as np
    E = np.concatenate([np.asarray(c[0], np.int32) for c in curves])
    G = np.concatenate([np.asarray(c[1], np.float64) for c in curves])
    cnt = np.array([len(c[0]) for c in curves], np.int32)
    off = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64)
    lz = np.zeros(len(curves))
    lp = np.zeros(len(curves))
    call("wlg_class_log_probs", E.ctypes.data_as(P), G.ctypes.data_as(P), off.ctypes.data_as(P),
         cnt.ctypes.data_as(P), len(curves), prob, lz.ctypes.data_as(P), lp.ctypes.data_as(P))
    return lz, lp


# ----------------------------------------------------------------- serving --

class ServerConfig(C.Structure):
    _fields_ = [("mem_budget_bytes", sz), ("epoch_outer", i32), ("max_prerun_batch", i32), ("max_resident", i32),
                ("fail_after_epochs", i32), ("stitching", i32), ("max_readmit", i32)]


class Decoded(C.Structure):
    """wlg_decoded: one retired request (classes in the order i, v, h, c)."""
    _fields_ = [("id", u64), ("status", i32), ("readmissions", i32), ("outer_iterations", i64 * 4), ("log_z", f64 * 4),
                ("log_probs", f64 * 4), ("submit_ms", f64), ("done_ms", f64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", i64), ("completed", i64), ("resident_problems", i64), ("epochs", i64),
                ("main_launches", i64), ("prerun_launches", i64), ("bytes_in_use", i64), ("bytes_budget", i64),
                ("readmitted", i64)]


class Server:
    """Continuous-batching decoder (wlg_server_*): submit disorder samples,
    poll retired requests with their four class log-probabilities."""

    def __init__(self, device: int = 0, mem_budget_bytes: int = 0, epoch_outer: int = 0, max_prerun_batch: int = 0,
                 max_resident: int = 0, fail_after_epochs: int = 0, stitching: int = 0, max_readmit: int = 0):
        cfg = ServerConfig(mem_budget_bytes, epoch_outer, max_prerun_batch, max_resident, fail_after_epochs, stitching,
                           max_readmit)
        h = C.c_void_p()
        call("wlg_server_create", device, C.byref(cfg), C.byref(h))
        self._h = h

    def submit(self, requests, couplings=None):
        """Queue requests (Problems; error_class ignored); returns their ids.  couplings: None (drawn)
        or one class-'i' bond pattern (+-1, 2*X*Y) per request (wlg_server_submit_couplings)."""
        n = len(requests)
        arr = (Problem * n)(*requests)
        ids = (u64 * max(n, 1))()
        J = _couplings(requests, couplings)
        self._check("wlg_server_submit_couplings",
                    lib().wlg_server_submit_couplings(self._h, C.cast(arr, P), n,
                                                      None if J is None else J.ctypes.data_as(P), C.cast(ids, P)))
        return [int(ids[i]) for i in range(n)]

    def poll(self, cap: int = 256, timeout_ms: int = 0):
        """Up to `cap` retired requests (Decoded), waiting up to timeout_ms for one."""
        out = (Decoded * cap)()
        k = i32(0)
        self._check("wlg_server_poll", lib().wlg_server_poll(self._h, C.cast(out, P), cap, C.byref(k), timeout_ms))
        return [out[i] for i in range(k.value)]

    def wait(self, ids, timeout_s: float = 600.0):
        """Poll until every id in `ids` is retired: {id: Decoded}."""
        import time
        want, got = set(ids), {}
        t_end = time.monotonic() + timeout_s
        while want - set(got):
            if time.monotonic() > t_end:
                raise TimeoutError(f"{len(want - set(got))} requests not retired")
            for d in self.poll(256, 100):
                got[int(d.id)] = d
        return {i: got[i] for i in ids}

    def stats(self):
        st = ServerStats()
        call("wlg_server_stats_get", self._h, C.byref(st))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def _check(self, name, st):
        if st != 0:
            detail = lib().wlg_server_last_error(self._h).decode()
            raise WlgError(name, st, f"{lib().wlg_status_string(st).decode()}: {detail}")

    def close(self):
        if self._h:
            lib().wlg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ HDF5 files --

H5_TYPES = {0: "u1", 1: "i1", 2: "<i4", 3: "<u8", 4: "<f8", 5: [("Key", "<i4"), ("pad", "<i4"), ("Value", "<f8")]}


def h5_list(path: str, group: str = ""):
    """Children of a group in a result file: (groups, datasets)."""
    buf = C.create_string_buffer(1 << 20)
    call("wlg_h5_list", path.encode(), group.encode(), C.cast(buf, P), len(buf))
    names = buf.value.decode().splitlines()
    return [n[:-1] for n in names if n.endswith("/")], [n for n in names if not n.endswith("/")]


def h5_read(path: str, dataset: str):
    """A dataset of a result file as a numpy array (compound: fields Key, Value)."""
    import numpy as np
    t, n = i32(0), u64(0)
    call("wlg_h5_read", path.encode(), dataset.encode(), C.byref(t), C.byref(n), None, 0)
    dt = np.dtype(H5_TYPES[t.value])
    out = np.zeros(n.value, dt)
    call("wlg_h5_read", path.encode(), dataset.encode(), C.byref(t), C.byref(n), out.ctypes.data_as(P), out.nbytes)
    return out


def h5_attribute(path: str, dataset: str, name: str) -> str:
    buf = C.create_string_buffer(4096)
    call("wlg_h5_attribute", path.encode(), dataset.encode(), name.encode(), C.cast(buf, P), len(buf))
    return buf.value.decode()
