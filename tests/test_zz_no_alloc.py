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

WLG_ERR_CAPACITY = 9


def _noalloc_raw(wlg, probs, res=None, raw_fill=0.0):
    n = len(probs)
    arr = (wlg.Problem * n)(*probs)
    if res is None:
        res = (wlg.Result * n)()
    n_win = sum(p.intervals for p in probs)
    ws = np.zeros(n_win, np.int32)
    we = np.zeros(n_win, np.int32)
    cap = sum(p.intervals * (4 * p.X * p.Y + 1) for p in probs)
    raw = np.full(cap, raw_fill, np.float64)
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


def _wide_window(wlg, k, max_outer=3):
    """16x16, one window of 96 walkers: about 192 bins x 96 walkers x 16 B of
    team state, above shared memory, so the main run keeps FP64 log g in the
    global pool (form 3)."""
    return wlg.problem(16, 16, prob=0.04, seed=12345, sample=k, pre_iterations=2000, intervals=1,
                       walkers_per_interval=96, max_outer=max_outer)


def test_noalloc_matches_allocating_solve_twice(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    first = [wlg.problem(6, 6, prob=0.04, error_class=c, seed=12345, sample=k, beta=0.01, iterations=500)
             for k in range(3) for c in "iv"]
    second = [wlg.problem(5, 4, boundary=1, prob=0.1, error_class="h", seed=9, sample=k, pre_walkers=64,
                          pre_intervals=12, pre_iterations=2000, intervals=5, walkers_per_interval=4, beta=0.02,
                          iterations=400, exchange_every=2) for k in range(4)]
    _compare(wlg, first)   # the arena holds whatever an earlier call (or nothing) left there
    _compare(wlg, second)  # the arena still holds the first call's buffers


def test_noalloc_global_pool_form_matches_allocating_solve(cuda):
    """A batch in the global-pool form that fits the arena, twice in a row."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = [_wide_window(wlg, k) for k in range(2)]
    ctx = wlg.Context(0)
    ctx.solve_raw(probs)
    assert ctx.stats()["main_forms"] == 1 << 3
    _compare(wlg, probs)
    _compare(wlg, probs)


def test_noalloc_bench_batch_fits(cuda):
    """The 6x6 periodic batch of 100 samples x 4 classes (pre-run 128 walkers,
    32 bins; main run 10 windows x 3 walkers) fits the arena."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = [wlg.problem(6, 6, prob=0.04, error_class=c, seed=12345, sample=k) for c in "ivhc" for k in range(100)]
    _compare(wlg, probs)


def _sentinel_results(wlg, n):
    res = (wlg.Result * n)()
    for r in res:
        r.status, r.new_energy, r.outer_iterations, r.flips, r.pre_flips = -77, -78, -79, -80, -81
        r.n_energies, r.offset = -82, -83
    return res


def _untouched(res):
    return all((r.status, r.new_energy, r.outer_iterations, r.flips, r.pre_flips, r.n_energies, r.offset)
               == (-77, -78, -79, -80, -81, -82, -83) for r in res)


def test_noalloc_rejects_batches_beyond_the_arena(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    big = [wlg.problem(24, 24, prob=0.1, sample=k, intervals=64, walkers_per_interval=8) for k in range(200)]
    res = _sentinel_results(wlg, len(big))
    st, res2, _, _, raw, _ = _noalloc_raw(wlg, big, res=res, raw_fill=7.0)
    assert st == WLG_ERR_CAPACITY  # before any work
    assert _untouched(res2) and np.all(raw == 7.0)


def test_noalloc_rejects_global_pool_overflow_before_any_work(cuda):
    """60 problems in the global-pool form: their pre-run, hand-off and result
    buffers take about 1 MiB, but one log g slice per resident team
    (192 bins x 96 walkers x 8 B each, about 8.4 MiB together) does not fit
    the 8 MiB arena.  The batch is refused before the pre-run runs: results
    and outputs keep what the caller put there."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = [_wide_window(wlg, k) for k in range(60)]
    res = _sentinel_results(wlg, len(probs))
    st, res2, _, _, raw, _ = _noalloc_raw(wlg, probs, res=res, raw_fill=7.0)
    assert st == WLG_ERR_CAPACITY
    assert _untouched(res2) and np.all(raw == 7.0)
    # the arena is still usable afterwards
    _compare(wlg, [_wide_window(wlg, 0)])
