"""wlg_solve_raw_noalloc: the solve for callers that cannot allocate device
memory (a framework owns the memory pool, a latency-critical loop, a
no-allocation-after-start-up policy).  Through the C ABI, two calls in a
row, each compared with the allocating entry point wlg_solve_raw on the
same problems; bit-exact is this suite's tolerance for the engine.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_raw(wlg, probs):
    n = len(probs)
    arr = (wlg.Problem * n)(*probs)
    res = (wlg.Result * n)()
    n_win = sum(p.intervals for p in probs)
    ws = np.zeros(n_win, np.int32)
    we = np.zeros(n_win, np.int32)
    cap = sum(p.intervals * (4 * p.X * p.Y + 1) for p in probs)
    raw = np.zeros(cap, np.float64)
    off = np.zeros(n, np.int64)
    st = wlg.lib().wlg_solve_raw_noalloc(C.cast(arr, C.c_void_p), n, C.cast(res, C.c_void_p),
                                         ws.ctypes.data_as(C.c_void_p), we.ctypes.data_as(C.c_void_p),
                                         raw.ctypes.data_as(C.c_void_p), cap, off.ctypes.data_as(C.c_void_p), None)
    return st, list(res), ws, we, raw, off


def _compare(wlg, probs):
    st, res, ws, we, raw, off = _noalloc_raw(wlg, probs)
    assert st == 0, wlg.lib().wlg_status_string(st)
    want = wlg.Context(0).solve_raw(probs)
    wpos = 0
    for p, (r_ref, s_ref, e_ref, wins_ref) in enumerate(want):
        r = res[p]
        assert (r.status, r.outer_iterations, r.flips) == (r_ref.status, r_ref.outer_iterations, r_ref.flips)
        I = probs[p].intervals
        assert np.array_equal(ws[wpos:wpos + I], s_ref) and np.array_equal(we[wpos:wpos + I], e_ref)
        wpos += I
        pos = int(off[p])
        for b, w in enumerate(wins_ref):
            assert np.array_equal(raw[pos:pos + len(w)], w), (p, b)
            pos += len(w)


def test_noalloc_matches_allocating_solve_twice(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    first = [wlg.problem(6, 6, prob=0.04, error_class=c, seed=12345, sample=k, beta=0.01, iterations=500)
             for k in range(3) for c in "iv"]
    second = [wlg.problem(5, 4, boundary=1, prob=0.1, error_class="h", seed=9, sample=k, pre_walkers=64,
                          pre_intervals=12, pre_iterations=2000, intervals=5, walkers_per_interval=4, beta=0.02,
                          iterations=400, exchange_every=2) for k in range(4)]
    _compare(wlg, first)   # the arena holds whatever an earlier call (or nothing) left there
    _compare(wlg, second)  # the arena still holds the first call's buffers


def test_noalloc_rejects_batches_beyond_the_arena(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    big = [wlg.problem(24, 24, prob=0.1, sample=k, intervals=64, walkers_per_interval=8) for k in range(200)]
    st, *_ = _noalloc_raw(wlg, big)
    assert st == 9  # WLG_ERR_CAPACITY, before any work
