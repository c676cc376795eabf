"""The batched engine (one pre-run CTA and one persistent main-run team per
problem) against the oracle's restatement of prerun.cu + mainrun.cu.

Every problem's trajectory is deterministic given (seed, sample), so the
walker-0 log g of every window must equal the oracle's bit for bit, and the
stitched, normalised result must equal the oracle's stitching of it.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def oracle_run(X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n, I, W, overlap, alpha, beta, n_iter, xc,
               xmode, gpar, max_outer=0):
    N = X * Y
    seen = np.zeros(R * (4 * N + 1), np.uint8)
    J = np.zeros(R * 2 * N, np.int8)
    flat = np.zeros(R * pre_i * N, np.int8)
    flag = np.zeros(R * pre_i, np.int32)
    en = np.zeros(R * pre_i, np.int32)
    L = O.lib()
    L.orc_prerun(X, Y, boundary, C.c_float(prob), cls.encode(), seed, R, pre_w, pre_i, pre_n, O.ptr(seen), O.ptr(J),
                 O.ptr(flat), O.ptr(flag), O.ptr(en))
    start = np.zeros(R * I, np.int32)
    end = np.zeros(R * I, np.int32)
    off_hist = np.zeros(R * I * W, np.int32)
    n_log = C.c_longlong(0)
    ci = np.zeros(R, np.int32)
    outer = C.c_longlong(0)
    flips = C.c_longlong(0)
    args = (X, Y, boundary, R, I, W, C.c_float(overlap), alpha, beta, n_iter, xc, xmode, gpar, seed,
            max_outer, O.ptr(seen), O.ptr(J), O.ptr(flat), O.ptr(flag), O.ptr(en), pre_i, O.ptr(start), O.ptr(end),
            O.ptr(off_hist))
    st = L.orc_mainrun(*args, None, C.byref(n_log), O.ptr(ci), C.byref(outer), C.byref(flips))
    logG = np.zeros(max(n_log.value, 1), np.float64)
    st = L.orc_mainrun(*args, O.ptr(logG), C.byref(n_log), O.ptr(ci), C.byref(outer), C.byref(flips))
    return dict(status=st, start=start, end=end, off_hist=off_hist, logG=logG, cond=ci, outer=outer.value,
                flips=flips.value)


CONFIGS = [
    # X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n, I, W, overlap, alpha, beta, n_iter, xc, xmode, gpar
    (4, 4, 0, 0.04, "i", 12345, 3, 32, 8, 2000, 10, 3, 0.25, 0.8, 0.001, 1000, 20, 1, 0),
    (4, 4, 0, 0.10, "c", 7, 4, 32, 8, 2000, 4, 3, 0.25, 0.8, 0.01, 500, 1, 0, 1),
    (5, 4, 1, 0.20, "h", 99, 3, 32, 9, 3000, 5, 2, 0.5, 0.8, 0.005, 400, 3, 1, 0),
    (6, 6, 0, 0.04, "v", 12345, 2, 128, 32, 2000, 10, 3, 0.25, 0.8, 0.01, 1000, 20, 1, 0),
    (5, 5, 1, 0.20, "i", 31337, 2, 64, 16, 3000, 7, 3, 0.25, 0.8, 0.01, 800, 2, 1, 1),
    (9, 8, 0, 0.08, "i", 5, 1, 64, 16, 3000, 8, 2, 0.25, 0.7, 0.05, 1500, 4, 1, 0),
]


@pytest.mark.parametrize("cfg", CONFIGS, ids=[f"{c[0]}x{c[1]}b{c[2]}{c[4]}" for c in CONFIGS])
def test_engine_full_run_bit_exact(cuda, cfg):
    import qec_pf_wang_landau_gb300 as wlg
    (X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n, I, W, overlap, alpha, beta, n_iter, xc, xmode,
     gpar) = cfg
    ref = oracle_run(*cfg)
    assert ref["status"] == 0
    probs = [wlg.problem(X, Y, boundary=boundary, prob=prob, error_class=cls, seed=seed, sample=k,
                         pre_walkers=pre_w, pre_intervals=pre_i, pre_iterations=pre_n, intervals=I,
                         walkers_per_interval=W, overlap=overlap, alpha=alpha, beta=beta, iterations=n_iter,
                         exchange_every=xc, exchange_mode=xmode, global_parity=gpar) for k in range(R)]
    ctx = wlg.Context(0)
    out = ctx.solve_raw(probs)
    total_flips = 0
    for k, (res, s, e, wins) in enumerate(out):
        assert res.status == 0, (k, res.status, res.new_energy)
        total_flips += res.flips
        assert np.array_equal(s, ref["start"][k * I:(k + 1) * I])
        assert np.array_equal(e, ref["end"][k * I:(k + 1) * I])
        for b in range(I):
            o = ref["off_hist"][(k * I + b) * W]
            want = ref["logG"][o:o + (e[b] - s[b] + 1)]
            assert np.array_equal(wins[b], want), f"sample {k} window {b}: max |d| {np.abs(wins[b] - want).max()}"
    assert total_flips == ref["flips"]

    # stitched result == the oracle's stitching of the same windows, in the
    # reference's mode (the default) and in the defined one
    for mode in (wlg.STITCH_DEFINED, wlg.STITCH_REFERENCE):
        ctx.set_stitching(mode)
        solved = ctx.solve(probs)
        for k, (res, E, G) in enumerate(solved):
            o = ref["off_hist"][k * I * W]
            sl = np.ascontiguousarray(ref["logG"][o:])
            Eo = np.zeros(4 * X * Y + 1, np.int32)
            Go = np.zeros(4 * X * Y + 1, np.float64)
            nout = C.c_int(0)
            rc = O.lib().orc_stitch(O.ptr(sl), O.ptr(ref["start"][k * I:]), O.ptr(ref["end"][k * I:]), I, W, X, Y,
                                    O.ptr(Eo), O.ptr(Go), len(Eo), C.byref(nout), mode)
            if rc != 0:
                assert res.status == 8, (mode, k, res.status)  # WLG_ERR_STITCH
                continue
            assert np.array_equal(E, Eo[:nout.value])
            assert np.array_equal(G, Go[:nout.value])
            lse = np.logaddexp.reduce(G)
            assert abs(lse - X * Y * np.log(2)) < 1e-9


# Problems whose per-team state (FP64 + float log g, histogram, lattices) is
# above 227 KB of shared memory: the main run keeps FP64 log g in a global
# pool (form 3).  Capped at three outer iterations; the cap ends both sides at
# the same point.
BIG = [
    # 16x16, one window of 96 walkers: 192 bins x 96 walkers x 16 B = 295 KB
    (16, 16, 0, 0.04, "i", 12345, 1, 128, 32, 2000, 1, 96, 0.25, 0.8, 1e-3, 1000, 20, 1, 0),
    # 20x20, two windows of 48 walkers exchanging every iteration: 212 bins x 96 walkers x 16 B = 326 KB
    (20, 20, 0, 0.04, "v", 12345, 1, 128, 32, 2000, 2, 48, 0.25, 0.8, 1e-3, 500, 1, 1, 0),
]


def big_problems(cfg, R=None, max_outer=3):
    import qec_pf_wang_landau_gb300 as wlg
    (X, Y, boundary, prob, cls, seed, R0, pre_w, pre_i, pre_n, I, W, overlap, alpha, beta, n_iter, xc, xmode,
     gpar) = cfg
    return [wlg.problem(X, Y, boundary=boundary, prob=prob, error_class=cls, seed=seed, sample=k,
                        pre_walkers=pre_w, pre_intervals=pre_i, pre_iterations=pre_n, intervals=I,
                        walkers_per_interval=W, overlap=overlap, alpha=alpha, beta=beta, iterations=n_iter,
                        exchange_every=xc, exchange_mode=xmode, global_parity=gpar, max_outer=max_outer)
            for k in range(R0 if R is None else R)]


@pytest.mark.parametrize("cfg", BIG, ids=[f"{c[0]}x{c[1]}I{c[10]}W{c[11]}" for c in BIG])
def test_engine_global_log_g_form_bit_exact(cuda, cfg):
    import qec_pf_wang_landau_gb300 as wlg
    I = cfg[10]
    ref = oracle_run(*cfg, max_outer=3)
    assert ref["status"] == 3 and ref["outer"] == 3
    ctx = wlg.Context(0)
    out = ctx.solve_raw(big_problems(cfg))
    assert ctx.stats()["main_forms"] == 1 << 3
    (res, s, e, wins), = out
    assert res.status == wlg.WLG_ERR_TIMEOUT and res.outer_iterations == 3
    assert res.flips == ref["flips"]
    assert np.array_equal(s, ref["start"][:I]) and np.array_equal(e, ref["end"][:I])
    for b in range(I):
        o = ref["off_hist"][b * cfg[11]]
        want = ref["logG"][o:o + (e[b] - s[b] + 1)]
        assert np.array_equal(wins[b], want), f"window {b}: max |d| {np.abs(wins[b] - want).max()}"


# Large lattices with the large-lattice workload's window layout: 64 windows
# x 8 walkers (512-thread teams), overlap 0.3, exchange every 10 iterations,
# p = 0.10; capped at two outer iterations.  24x24 runs in the global-pool
# form, 16x16 in shared memory.
LARGE = [
    (24, 24, 0, 0.10, "h", 4242, 1, 128, 128, 57600, 64, 8, 0.3, 0.8, 1e-8, 1000, 10, 1, 0),
    (16, 16, 0, 0.10, "c", 4242, 1, 128, 128, 25600, 64, 8, 0.3, 0.8, 1e-8, 1000, 10, 1, 0),
]


@pytest.mark.parametrize("cfg", LARGE, ids=[f"{c[0]}x{c[1]}I{c[10]}W{c[11]}" for c in LARGE])
def test_engine_large_teams_bit_exact(cuda, cfg):
    import qec_pf_wang_landau_gb300 as wlg
    I, W = cfg[10], cfg[11]
    ref = oracle_run(*cfg, max_outer=2)
    assert ref["status"] == 3
    ctx = wlg.Context(0)
    (res, s, e, wins), = ctx.solve_raw(big_problems(cfg, max_outer=2))
    assert res.status == wlg.WLG_ERR_TIMEOUT and res.flips == ref["flips"]
    assert np.array_equal(s, ref["start"][:I]) and np.array_equal(e, ref["end"][:I])
    for b in range(I):
        o = ref["off_hist"][b * W]
        want = ref["logG"][o:o + (e[b] - s[b] + 1)]
        assert np.array_equal(wins[b], want), f"window {b}: max |d| {np.abs(wins[b] - want).max()}"


def test_engine_mixed_forms_batch_equals_separate_runs(cuda):
    """A batch holding shared-memory-form and global-pool-form problems (two
    persistent launches, one global pool) gives each problem its result alone."""
    import qec_pf_wang_landau_gb300 as wlg
    small = wlg.problem(6, 6, prob=0.04, error_class="h", seed=12345, sample=3, max_outer=3)
    batch = [big_problems(BIG[1])[0], small, big_problems(BIG[0])[0]]
    ctx = wlg.Context(0)
    together = ctx.solve_raw(batch)
    assert ctx.stats()["main_forms"] & (1 << 3) and ctx.stats()["main_forms"] != 1 << 3
    for p, (r, s, e, wins) in zip(batch, together):
        (r1, s1, e1, wins1), = ctx.solve_raw([p])
        assert r.status == r1.status and r.flips == r1.flips and r.outer_iterations == r1.outer_iterations
        assert np.array_equal(s, s1) and np.array_equal(e, e1)
        assert all(np.array_equal(a, b) for a, b in zip(wins, wins1))


def random_configs(n, seed=20261203):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        X, Y = int(rng.integers(3, 10)), int(rng.integers(3, 10))
        I = int(rng.integers(2, 9))
        out.append((X, Y, int(rng.integers(0, 2)), float(np.float32(rng.uniform(0.02, 0.2))), "ivhc"[rng.integers(0, 4)],
                    int(rng.integers(1, 10 ** 6)), 1, 64, 16, 2000, I, int(rng.integers(1, 6)),
                    float(rng.choice([0.2, 0.25, 0.5])), 0.8, 0.02, int(rng.integers(200, 1001)),
                    int(rng.choice([1, 2, 5, 20])), int(rng.integers(0, 2)), int(rng.integers(0, 2))))
    return out


def test_engine_random_configs_bit_exact_in_one_batch(cuda):
    """Seeded random problems (size, boundary, class, p, windows, walkers,
    overlap, n, exchange cadence, mode and parity) in one heterogeneous batch:
    each equals the oracle's run of it alone, capped at 6 outer iterations."""
    import qec_pf_wang_landau_gb300 as wlg
    cfgs = random_configs(12)
    refs = [oracle_run(*c, max_outer=6) for c in cfgs]
    probs = [big_problems(c, max_outer=6)[0] for c in cfgs]
    out = wlg.Context(0).solve_raw(probs)
    compared = 0
    for c, ref, (res, s, e, wins) in zip(cfgs, refs, out):
        I, W = c[10], c[11]
        if ref["status"] not in (0, 3):
            assert res.status != 0, c  # the oracle's run stopped on a new energy or had no lattice
            continue
        assert res.status == (0 if ref["status"] == 0 else wlg.WLG_ERR_TIMEOUT), c
        assert res.flips == ref["flips"], c
        assert np.array_equal(s, ref["start"][:I]) and np.array_equal(e, ref["end"][:I]), c
        for b in range(I):
            o = ref["off_hist"][b * W]
            assert np.array_equal(wins[b], ref["logG"][o:o + (e[b] - s[b] + 1)]), (c, b)
        compared += 1
    assert compared >= 8


EDGE = [
    # two rows: the up and down neighbours of a site coincide (periodic), or one is missing (open)
    (2, 5, 0, 0.1, "i", 11, 2, 32, 8, 2000, 3, 3, 0.25, 0.8, 1e-3, 500, 1, 1, 0),
    (2, 2, 1, 0.2, "h", 12, 2, 32, 4, 1000, 2, 2, 0.5, 0.8, 1e-3, 300, 1, 1, 0),
    (5, 2, 1, 0.1, "c", 13, 1, 32, 8, 2000, 3, 2, 0.25, 0.8, 1e-3, 300, 2, 1, 0),
    # the largest lattice (4096 spins; 16 pre-run walkers fit one SM's shared memory)
    (64, 64, 0, 0.05, "i", 21, 1, 16, 16, 2000, 4, 8, 0.25, 0.8, 1e-3, 100, 1, 1, 0),
]


@pytest.mark.parametrize("cfg", EDGE, ids=[f"{c[0]}x{c[1]}b{c[2]}" for c in EDGE])
def test_edge_lattices_bit_exact(cuda, cfg):
    """Two-row lattices and the maximum size against the oracle's run, capped
    at 2 outer iterations: per-window log g and move counts bit for bit."""
    import qec_pf_wang_landau_gb300 as wlg
    I, W = cfg[10], cfg[11]
    ref = oracle_run(*cfg, max_outer=2)
    assert ref["status"] == 3, ref["status"]  # ran until the cap
    out = wlg.Context(0).solve_raw(big_problems(cfg, max_outer=2))
    assert sum(r.flips for r, _, _, _ in out) == ref["flips"]
    for k, (res, s, e, wins) in enumerate(out):
        assert res.status == wlg.WLG_ERR_TIMEOUT
        assert np.array_equal(s, ref["start"][k * I:(k + 1) * I]) and np.array_equal(e, ref["end"][k * I:(k + 1) * I])
        for b in range(I):
            o = ref["off_hist"][(k * I + b) * W]
            assert np.array_equal(wins[b], ref["logG"][o:o + (e[b] - s[b] + 1)]), (k, b)


def test_empty_batch(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    ctx = wlg.Context(0)
    assert ctx.solve([]) == []
    assert ctx.solve_raw([]) == []
    with wlg.Server(0) as srv:
        assert srv.submit([]) == []


def test_engine_heterogeneous_batch_equals_separate_runs(cuda):
    """Problems of different shapes in one batch give the same results as alone."""
    import qec_pf_wang_landau_gb300 as wlg
    mk = lambda X, Y, b, k, c: wlg.problem(X, Y, boundary=b, prob=0.08, error_class=c, seed=4242, sample=k,
                                           pre_walkers=64, pre_intervals=16, pre_iterations=2000, intervals=6,
                                           walkers_per_interval=4, beta=0.02, iterations=600, exchange_every=2)
    batch = [mk(4, 4, 0, 0, "i"), mk(6, 6, 0, 1, "v"), mk(5, 7, 1, 2, "h"), mk(8, 8, 0, 3, "c"), mk(9, 9, 1, 4, "i")]
    ctx = wlg.Context(0)
    together = ctx.solve(batch)
    for p, (r, E, G) in zip(batch, together):
        (r1, E1, G1), = ctx.solve([p])
        assert r.status == r1.status == 0
        assert r.flips == r1.flips and r.outer_iterations == r1.outer_iterations
        assert np.array_equal(E, E1) and np.array_equal(G, G1)


def test_autotune_picks_teams_per_cta_without_changing_results(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    probs = [wlg.problem(6, 6, prob=0.04, error_class=c, seed=99, sample=k, beta=0.01, iterations=500)
             for k in range(12) for c in "ivhc"] + \
            [wlg.problem(9, 9, prob=0.05, error_class="i", seed=99, sample=k, intervals=8, walkers_per_interval=6,
                         beta=0.05, iterations=400) for k in range(4)]
    ctx = wlg.Context(0)
    before = ctx.solve(probs)
    tuned = ctx.autotune(probs, max_outer=2)
    assert len(tuned) == 2  # (form 2, 32 threads) and (form 0, 64 threads)
    for t in tuned:
        assert t["candidates"] >= 1 and 1 <= t["per_cta"] <= 256 // t["team"] and t["main_ms"] > 0
    after = ctx.solve(probs)
    for (r1, E1, G1), (r2, E2, G2) in zip(before, after):
        assert r1.status == r2.status and r1.outer_iterations == r2.outer_iterations
        assert np.array_equal(E1, E2) and np.array_equal(G1, G2)


def test_solve_on_a_caller_stream(cuda):
    """wlg_context_set_stream: solves run on the caller's stream with the same results."""
    import qec_pf_wang_landau_gb300 as wlg
    torch = cuda
    probs = [wlg.problem(5, 5, prob=0.05, error_class=c, seed=3, sample=k, intervals=6, beta=0.02, iterations=500)
             for k in range(4) for c in "iv"]
    ctx = wlg.Context(0)
    a = ctx.solve(probs)
    s = torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)
    b = ctx.solve(probs)
    ctx.set_stream(None)
    c = ctx.solve(probs)
    for (r1, E1, G1), (r2, E2, G2), (r3, E3, G3) in zip(a, b, c):
        assert r1.status == r2.status == r3.status
        assert np.array_equal(G1, G2) and np.array_equal(G1, G3) and np.array_equal(E1, E2)


def test_engine_4x4_log_g_against_exact_enumeration(cuda):
    """Config 1 (4x4 periodic, p=0.04, seed 12345, class i): the normalised log g
    against exact FP64 enumeration of all 2^16 states."""
    import qec_pf_wang_landau_gb300 as wlg
    p = wlg.problem(4, 4, prob=0.04, error_class="i", seed=12345, sample=0, pre_walkers=32, pre_intervals=8,
                    pre_iterations=1000, intervals=10, walkers_per_interval=3, overlap=0.25, alpha=0.8, beta=1e-3,
                    iterations=1000, exchange_every=20)
    ctx = wlg.Context(0)
    (r, E, G), = ctx.solve([p])
    assert r.status == 0
    J = O.init_interactions(4, 4, 1, 12345, 0.04, "i")
    counts = O.exact_counts(J, 4, 4, 0)
    exact_E = np.nonzero(counts)[0] - 32
    assert set(E.tolist()) == set(exact_E.tolist())
    exact = np.log(counts[E + 32])
    err = G - exact
    assert np.sqrt(np.mean(err ** 2)) < 0.25
    assert np.abs(err).max() < 0.6


@pytest.mark.parametrize("boundary", [0, 1])
def test_engine_8x8_log_g_and_class_probabilities_against_exact(cuda, boundary):
    """8x8 (2^64 states) by the oracle's transfer matrix: the engine's stitched
    log g has exactly the reachable energies and WL-size errors, and the four
    class probabilities at the Nishimori temperature match the exact ones."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = [wlg.problem(8, 8, boundary=boundary, prob=0.08, error_class=c, seed=31, sample=0, pre_walkers=128,
                         pre_intervals=32, pre_iterations=6400, intervals=8, walkers_per_interval=4, beta=1e-4,
                         iterations=1000, exchange_every=5) for c in "ivhc"]
    out = wlg.Context(0).solve(probs)
    assert all(r.status == 0 for r, _, _ in out)
    exact_lz = []
    bn = 0.5 * np.log(0.92 / 0.08)
    for (r, E, G), c in zip(out, "ivhc"):
        J = O.init_interactions(8, 8, 1, 31, 0.08, c)
        cnt = O.exact_counts(J, 8, 8, boundary)
        assert set(E.tolist()) == set((np.nonzero(cnt)[0] - 128).tolist())
        err = G - np.log(cnt[E + 128])
        assert np.sqrt(np.mean(err ** 2)) < 0.5 and np.abs(err).max() < 1.5
        Ee = np.nonzero(cnt)[0] - 128
        exact_lz.append(np.logaddexp.reduce(np.log(cnt[Ee + 128]) - bn * Ee))
    exact_lp = np.array(exact_lz) - np.logaddexp.reduce(exact_lz)
    _, lp = wlg.class_log_probs([(E, G) for _, E, G in out], 0.08)
    assert np.abs(np.exp(lp) - np.exp(exact_lp)).max() < 0.05


def test_engine_10x10_against_exact_and_oracle(cuda):
    """10x10 (2^100 states, two 64-bit words of spins per walker), periodic
    and open, all four classes in one batch: every stitched curve has exactly
    the reachable energies and WL-size errors against the transfer matrix,
    the class probabilities match the exact ones (on the open lattice every
    class is a gauge copy of i: exactly 1/4 each), and the periodic class-i
    run equals the oracle's bit for bit."""
    import qec_pf_wang_landau_gb300 as wlg
    X = Y = 10
    N = X * Y
    kw = dict(prob=0.08, seed=31, sample=0, pre_walkers=128, pre_intervals=32, pre_iterations=10000, intervals=12,
              walkers_per_interval=4, overlap=0.25, alpha=0.8, beta=1e-4, iterations=1000, exchange_every=5)
    probs = [wlg.problem(X, Y, boundary=b, error_class=c, **kw) for b in (0, 1) for c in "ivhc"]
    out = wlg.Context(0).solve(probs)
    assert all(r.status == 0 for r, _, _ in out)
    bn = 0.5 * np.log(0.92 / 0.08)
    for b in (0, 1):
        exact_lz = []
        for ci, c in enumerate("ivhc"):
            _, E, G = out[4 * b + ci]
            cnt = O.exact_counts(O.init_interactions(X, Y, 1, 31, 0.08, c), X, Y, b)
            Ee = np.nonzero(cnt)[0] - 2 * N
            assert set(E.tolist()) == set(Ee.tolist())
            err = G - np.log(cnt[E + 2 * N])
            assert np.sqrt(np.mean(err ** 2)) < 0.3 and np.abs(err).max() < 0.8
            exact_lz.append(np.logaddexp.reduce(np.log(cnt[Ee + 2 * N]) - bn * Ee))
        exact_lp = np.array(exact_lz) - np.logaddexp.reduce(exact_lz)
        if b == 1:
            assert np.allclose(np.exp(exact_lp), 0.25, atol=1e-12)
        _, lp = wlg.class_log_probs([(E, G) for _, E, G in out[4 * b:4 * b + 4]], 0.08)
        assert np.abs(np.exp(lp) - np.exp(exact_lp)).max() < 0.05
    ref = oracle_run(X, Y, 0, 0.08, "i", 31, 1, 128, 32, 10000, 12, 4, 0.25, 0.8, 1e-4, 1000, 5, 1, 0)
    rc, Er, Gr = O.stitch(ref["logG"], ref["start"], ref["end"], 12, 4, X, Y)
    assert ref["status"] == 0 and rc == 0
    _, E, G = out[0]
    assert np.array_equal(E, Er) and np.array_equal(G, Gr)


def test_class_log_probs_normalised(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    probs = [wlg.problem(4, 4, prob=0.1, error_class=c, seed=77, sample=0, pre_walkers=32, pre_intervals=8,
                         pre_iterations=2000, intervals=4, walkers_per_interval=3, beta=0.01, iterations=500)
             for c in "ivhc"]
    ctx = wlg.Context(0)
    out = ctx.solve(probs)
    assert all(r.status == 0 for r, _, _ in out)
    lz, lp = wlg.class_log_probs([(E, G) for _, E, G in out], 0.1)
    assert abs(np.logaddexp.reduce(lp)) < 1e-12
    # exact class probabilities from enumeration agree to WL accuracy
    exact = []
    for c in "ivhc":
        J = O.init_interactions(4, 4, 1, 77, 0.1, c)
        cnt = O.exact_counts(J, 4, 4, 0)
        Ee = np.nonzero(cnt)[0] - 32
        bn = 0.5 * np.log(0.9 / 0.1)
        exact.append(np.logaddexp.reduce(np.log(cnt[Ee + 32]) - bn * Ee))
    exact = np.array(exact) - np.logaddexp.reduce(exact)
    assert np.argmax(lp) == np.argmax(exact)
    assert np.abs(np.exp(lp) - np.exp(exact)).max() < 0.05


@pytest.mark.parametrize("cls,xc,xmode,gpar,I", [("i", 20, 1, 0, 10), ("c", 1, 0, 1, 7), ("h", 3, 1, 1, 5)])
def test_plain_form_equals_batched_form(cuda, cls, xc, xmode, gpar, I):
    """The reference-structured plain form and the persistent batched form
    compute identical results (same streams, same FP64 operation order)."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = [wlg.problem(6, 6, prob=0.04, error_class=cls, seed=2024, sample=k, pre_walkers=128, pre_intervals=32,
                         pre_iterations=1000, intervals=I, walkers_per_interval=3, beta=0.01, iterations=500,
                         exchange_every=xc, exchange_mode=xmode, global_parity=gpar) for k in range(6)]
    plain, launches = wlg.solve_plain(probs)
    batched = wlg.Context(0).solve(probs)
    assert launches > 10
    for (r1, E1, G1), (r2, E2, G2) in zip(plain, batched):
        assert r1.status == r2.status == 0
        assert r1.outer_iterations == r2.outer_iterations and r1.flips == r2.flips
        assert np.array_equal(E1, E2) and np.array_equal(G1, G2)


def test_full_bench_workload_properties(cuda):
    """The bench workload at its full size (6x6 periodic, p = 0.04, 100 samples
    x 4 classes): every problem converges; every stitched log g has exactly the
    energies the lattice can reach (exact transfer-matrix counts) and
    logsumexp = N ln 2; each sample's four class probabilities sum to 1."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = [wlg.problem(6, 6, prob=0.04, error_class=c, seed=12345, sample=k, pre_walkers=128, pre_intervals=32,
                         pre_iterations=1000, intervals=10, walkers_per_interval=3, overlap=0.25, alpha=0.8,
                         beta=1e-3, iterations=1000, exchange_every=20, exchange_mode=1)
             for k in range(100) for c in "ivhc"]
    out = wlg.Context(0).solve(probs)
    assert all(r.status == 0 for r, _, _ in out)
    J = {c: O.init_interactions(6, 6, 100, 12345, 0.04, c) for c in "ivhc"}
    for q, (r, E, G) in enumerate(out):
        k, c = divmod(q, 4)
        cnt = O.exact_counts(J["ivhc"[c]][k * 72:(k + 1) * 72], 6, 6, 0)
        assert set(E.tolist()) == set((np.nonzero(cnt)[0] - 72).tolist()), q
        assert abs(np.logaddexp.reduce(G) - 36 * np.log(2)) < 1e-9
    for k in range(100):
        _, lp = wlg.class_log_probs([(E, G) for _, E, G in out[4 * k:4 * k + 4]], 0.04)
        assert abs(np.logaddexp.reduce(lp)) < 1e-12


@pytest.mark.parametrize("what", ["couplings", "lattice"])
def test_mainrun_entry_refuses_values_other_than_pm1(cuda, what):
    """wlg_mainrun (main run from pre-run data) checks the caller's couplings
    and stored lattices before any device work: a value other than +-1 is
    WLG_ERR_INVALID with the problem named."""
    import qec_pf_wang_landau_gb300 as wlg
    X = Y = 4
    N = X * Y
    q = wlg.problem(X, Y, pre_walkers=1, pre_intervals=1, pre_iterations=0, intervals=2, walkers_per_interval=2)
    probs = (wlg.Problem * 1)(q)
    seen = np.ones(4 * N + 1, np.uint8)
    J = np.ones(2 * N, np.int8)
    lat = -np.ones(N, np.int8)
    (J if what == "couplings" else lat)[5] = 0
    found = np.ones(1, np.int32)
    energy = np.array([-2 * N], np.int32)
    res = (wlg.Result * 1)()
    E = np.zeros(4 * N + 1, np.int32)
    G = np.zeros(4 * N + 1)
    ctx = wlg.Context(0)
    st = wlg.lib().wlg_mainrun(ctx._h, C.cast(probs, C.c_void_p), 1, O.ptr(seen), O.ptr(J), O.ptr(found),
                               O.ptr(energy), O.ptr(lat), 60.0, C.cast(res, C.c_void_p), O.ptr(E), O.ptr(G), len(E))
    assert st == 1 and "problem 0 not +-1" in wlg.lib().wlg_context_last_error(ctx._h).decode()


def test_main_times_bound_the_main_run(cuda):
    """wlg_last_main_times: every problem that ran its main run has
    0 <= start <= end on the device clock, the first start is 0 and the last
    end lies within the main run's event-timed duration; a problem refused at
    the hand-off (no stored lattice for a window) reports -1."""
    import qec_pf_wang_landau_gb300 as wlg
    refused = wlg.problem(6, 6, prob=0.08, seed=100, sample=3, pre_walkers=16, pre_intervals=16, pre_iterations=300,
                          intervals=14, walkers_per_interval=2, overlap=0.8)
    ok = [wlg.problem(X, X, boundary=b, seed=7, sample=k, beta=0.01, iterations=400)
          for k, (X, b) in enumerate([(4, 0), (6, 1), (5, 0), (8, 0)])]
    probs = ok[:2] + [refused] + ok[2:]
    ctx = wlg.Context(0)
    out = ctx.solve(probs)
    t0, t1 = ctx.main_times()
    assert len(t0) == len(probs)
    assert out[2][0].status == 5 and t0[2] == -1 and t1[2] == -1  # WLG_ERR_NO_LATTICE
    ran = [i for i in range(len(probs)) if i != 2]
    assert all(out[i][0].status == 0 for i in ran)
    assert all(0 <= t0[i] <= t1[i] for i in ran)
    assert min(t0[i] for i in ran) == 0.0
    main_ms = ctx.stats()["main_ms"]
    assert max(t1[i] for i in ran) <= main_ms * 1.01 + 0.05
