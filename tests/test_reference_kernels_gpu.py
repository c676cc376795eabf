"""Bit parity with the reference's OWN kernels (src/wl.cu compiled unmodified
into a cubin, launched by oracle/ref_harness.cu with the geometry of its
drivers), the engine's operators and the oracle, all three on identical
state in the reference's layout.  Every array must be equal bit for bit
after every operation: lattices, energies, histograms, FP64 log g, RNG
offsets, exchange permutations, lattice offsets, flags.

The reference is deterministic wherever these tests use it:
* the WL step and replica exchange: each thread owns its walker; windows are
  kept unfinished (ln f never reaches the final value within the test), so
  the reference's converged-window branch (Q5) is not entered, and every
  start spectrum is the exact one, so no energy lies outside the mask (Q6);
* window averaging with at most two walkers per window: two FP64 atomic
  additions onto 0 give the same sum in either order;
* the pre-run with one walker per sample: the histogram and the lattice store
  are not shared.
Non-flat log g makes rejections, steps that leave the window
(wl.cu:1108-1110) and exchange rejections happen; the tests check that they
did.
"""
import numpy as np
import pytest

import oracle as O
from tests.helpers import (Dev, assert_state_equal, copy_state, mainrun_state, o_average, o_check_histogram,
                           o_exchange, o_reset_finish, o_wang_landau, prerun_outputs)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(cuda):
    L = O.reference_harness()
    if L is None:
        pytest.skip("reference cubin not available on this machine")
    return L


# ------------------------------------------------- reference kernel calls --

def r_wang_landau(L, d, n_iter, seed):
    s = d.st
    T = s["R"] * s["I"] * s["W"]
    assert L.refh_k_wang_landau(d.p("lattice"), d.p("J"), d.p("H"), d.p("logG"), d.p("factor"), d.p("E"),
                                d.p("newE"), d.p("off_iter"), d.p("found"), d.p("start"), d.p("end"), d.p("off_hist"),
                                d.p("off_lat"), d.p("cond"), d.p("spectrum"), d.p("off_spec"), d.p("cond_inter"),
                                s["X"], s["Y"], n_iter, T, s["I"], s["I"] * s["W"], seed, s["boundary"]) == 0


def r_check_histogram(L, d, alpha):
    s = d.st
    T = s["R"] * s["I"] * s["W"]
    assert L.refh_k_check_histogram(d.p("H"), d.p("factor"), d.p("cond"), d.p("off_hist"), d.p("end"), d.p("start"),
                                    d.p("spectrum"), d.p("off_spec"), d.p("cond_inter"), alpha, T, s["I"] * s["W"],
                                    s["I"]) == 0


def r_average(L, d):
    s = d.st
    assert L.refh_k_average_log_g(d.p("logG"), d.p("start"), d.p("end"), d.p("spectrum"), d.p("cond"),
                                  d.p("off_hist"), d.p("off_spec"), d.p("cond_inter"), s["R"], s["W"], s["I"]) == 0


def r_reset_finish(L, d, beta):
    s = d.st
    assert L.refh_k_reset_cond(d.p("cond"), d.p("factor"), s["R"] * s["I"], beta, s["W"], s["R"], s["I"]) == 0
    assert L.refh_k_check_finished(d.p("cond_inter"), d.p("cond"), s["I"], s["R"]) == 0


def r_exchange(L, d, even, seed):
    s = d.st
    assert L.refh_k_replica_exchange(d.p("off_lat"), d.p("E"), d.p("perm"), d.p("off_iter"), d.p("start"),
                                     d.p("end"), d.p("off_hist"), d.p("cond_inter"), d.p("logG"), int(even), seed,
                                     s["I"], s["I"] * s["W"], s["R"] * s["I"]) == 0


# ----------------------------------------------------------------- states --

def exact_state(X, Y, boundary, prob, cls, seed, R, I, W, overlap):
    """The main run's start state from the oracle's pre-run (= the engine's),
    checked to hold every sample's exact spectrum."""
    pre = prerun_outputs(X, Y, boundary, prob, cls, seed, R, 64, 16, 4000)
    N = X * Y
    for k in range(R):
        cnt = O.exact_counts(pre["J"][k * 2 * N:(k + 1) * 2 * N], X, Y, boundary)
        seen = pre["seen"][k * (4 * N + 1):(k + 1) * (4 * N + 1)]
        assert np.array_equal(seen != 0, cnt != 0), "pre-run missed an energy; pick other parameters"
    return mainrun_state(pre, I, W, overlap)


def sqrt_chain(n):
    f = [np.e]
    for _ in range(n - 1):
        f.append(np.sqrt(f[-1]))
    return np.array(f)


def roughen(st, rng):
    """Non-flat log g and histograms, a different modification factor per window."""
    st["logG"][:] = rng.normal(0.0, 1.5, st["logG"].shape)
    st["H"][:] = rng.integers(0, 40, st["H"].shape).astype(np.uint64)
    chain = sqrt_chain(8)
    f = chain[rng.integers(0, len(chain), st["R"] * st["I"])]
    st["factor"][:] = np.repeat(f, st["W"])


class Trio:
    """The same state three times: reference kernels (device), engine
    operators (device), oracle (host)."""

    def __init__(self, torch, L, st):
        self.L = L
        self.r = Dev(torch, st)
        self.e = Dev(torch, st)
        self.o = copy_state(st)

    def check(self, where):
        snap_r = self.r.snapshot()
        assert_state_equal(snap_r, self.o, f"{where} (reference kernels vs oracle)")
        assert_state_equal(self.e.snapshot(), self.o, f"{where} (engine vs oracle)")
        return snap_r

    def wang_landau(self, n, seed):
        r_wang_landau(self.L, self.r, n, seed)
        self.e.wang_landau(n, seed)
        o_wang_landau(self.o, n, seed)

    def check_histogram(self, alpha):
        r_check_histogram(self.L, self.r, alpha)
        self.e.check_histogram(alpha)
        o_check_histogram(self.o, alpha)

    def average(self):
        r_average(self.L, self.r)
        self.e.average()
        o_average(self.o)

    def reset_finish(self, beta):
        r_reset_finish(self.L, self.r, beta)
        self.e.reset_finish(beta)
        o_reset_finish(self.o, beta)

    def exchange(self, even, seed):
        r_exchange(self.L, self.r, even, seed)
        self.e.exchange(even, seed, global_parity=1)  # the reference's parity (Q9)
        o_exchange(self.o, even, seed, global_parity=1)


def walker_moves(before, after, N):
    """Per walker after a one-step sweep: (accepted, rejected, left its window).
    An in-window step takes two draws (site, acceptance), a step that leaves
    the window one; an accepted step flips a spin of the walker's lattice."""
    draws = after["off_iter"].astype(np.int64) - before["off_iter"].astype(np.int64)
    T = len(draws)
    changed = np.array([not np.array_equal(after["lattice"][o:o + N], before["lattice"][o:o + N])
                        for o in before["off_lat"][:T]])
    return changed, (draws == 2) & ~changed, draws == 1


def exchange_counts(before, after, st, even):
    """(attempts, accepted swaps) of one exchange pass: thread 0 of an active
    window draws W-1 shuffle numbers; every walker whose pair lies in both
    windows draws one more; an accepted swap moves two lattice offsets."""
    R, I, W = st["R"], st["I"], st["W"]
    draws = after["off_iter"].astype(np.int64) - before["off_iter"].astype(np.int64)
    active = sum(1 for b in range(R * I) if b % I != I - 1 and (b % 2 == 0) == even
                 and before["cond_inter"][b // I] != -1)
    attempts = int(draws.sum()) - (W - 1) * active
    swaps = int(np.sum(after["off_lat"] != before["off_lat"])) // 2
    return attempts, swaps


# ------------------------------------------------------------------ tests --

LOOP = [
    # X, Y, boundary, prob, class, seed, R, I, W, overlap
    (4, 4, 0, 0.04, "i", 12345, 3, 6, 2, 0.25),
    (6, 6, 0, 0.04, "v", 777, 2, 5, 2, 0.25),
    (5, 4, 1, 0.15, "h", 31, 3, 5, 2, 0.3),
    (6, 5, 1, 0.1, "c", -9, 2, 4, 1, 0.25),
]


@pytest.mark.parametrize("cfg", LOOP, ids=[f"{c[0]}x{c[1]}b{c[2]}{c[4]}I{c[7]}W{c[8]}" for c in LOOP])
def test_main_loop_replay_equals_reference_kernels(cuda, ref, cfg):
    """mainrun.cu:243-371 step by step: WL sweep, flatness, averaging, reset,
    finished check, exchange of both parities every outer iteration; every
    array equal after every operation."""
    X, Y, boundary, prob, cls, seed, R, I, W, overlap = cfg
    st = exact_state(X, Y, boundary, prob, cls, seed, R, I, W, overlap)
    t = Trio(cuda, ref, st)
    t.check("start")
    left = moved = swaps = 0
    n = 300
    for outer in range(10):
        before = t.r.snapshot()
        t.wang_landau(n, seed)
        after = t.check(f"outer {outer}: wang_landau")
        # per walker: n proposals; in-window steps draw twice, steps leaving the window once
        draws = after["off_iter"].astype(np.int64) - before["off_iter"].astype(np.int64)
        left += int(np.sum(2 * n - draws))
        moved += int(np.sum(after["E"] != before["E"]))
        t.check_histogram(0.8)
        t.check(f"outer {outer}: check_histogram")
        t.average()
        t.check(f"outer {outer}: average")
        t.reset_finish(1e-6)
        snap = t.check(f"outer {outer}: reset/finished")
        assert not np.any(snap["cond"] == 1)  # no window finishes: ln f > 1e-6 throughout
        for even in (True, False):
            t.exchange(even, seed)
            after_x = t.check(f"outer {outer}: exchange even={even}")
            swaps += exchange_counts(snap, after_x, st, even)[1]
            snap = after_x
    assert left > 0 and moved > 0 and swaps > 0, (left, moved, swaps)


@pytest.mark.parametrize("W", [3, 5])
@pytest.mark.parametrize("boundary", [0, 1])
def test_wang_landau_step_from_rough_state(cuda, ref, W, boundary):
    """wl.cu:1033-1130 from non-flat log g and histograms, a different ln f per
    window, W walkers per window: rejections and out-of-window steps on every
    sweep."""
    rng = np.random.default_rng(100 + W + 10 * boundary)
    st = exact_state(6, 6, boundary, 0.1, "i", 4242, 3, 6, W, 0.25)
    roughen(st, rng)
    t = Trio(cuda, ref, st)
    acc = rej = left = 0
    for rep in range(12):
        before = t.r.snapshot()
        t.wang_landau(1, 4242)
        after = t.check(f"step {rep}")
        a, r, l = walker_moves(before, after, st["N"])
        acc, rej, left = acc + int(a.sum()), rej + int(r.sum()), left + int(l.sum())
    assert acc > 0 and rej > 0 and left > 0, (acc, rej, left)
    for rep in range(3):
        t.wang_landau(500, 4242)
        t.check(f"sweep {rep}")


@pytest.mark.parametrize("W", [3, 4])
def test_replica_exchange_from_rough_state(cuda, ref, W):
    """wl.cu:785-890 with its Fisher-Yates draws, both parities, repeatedly,
    after sweeps that spread the walkers over their windows; rough log g makes
    some swaps fail."""
    rng = np.random.default_rng(7 * W)
    st = exact_state(6, 6, 0, 0.04, "h", 99, 2, 5, W, 0.4)
    roughen(st, rng)
    t = Trio(cuda, ref, st)
    attempts = swaps = 0
    for rep in range(6):
        t.wang_landau(200, 99)
        snap = t.check(f"rep {rep}: sweep")
        for even in (True, False):
            t.exchange(even, 99)
            after = t.check(f"rep {rep}: exchange even={even}")
            a, s_ = exchange_counts(snap, after, st, even)
            attempts, swaps = attempts + a, swaps + s_
            snap = after
    assert 0 < swaps < attempts, (swaps, attempts)  # swaps accepted and rejected


def test_check_histogram_flat_and_rough_windows(cuda, ref):
    """wl.cu:892-967 on windows that are flat for all walkers, for some, or for none."""
    rng = np.random.default_rng(5)
    st = exact_state(6, 6, 0, 0.04, "i", 5, 3, 8, 3, 0.25)
    roughen(st, rng)
    H = st["H"]
    for b in range(st["R"] * st["I"]):
        kind = b % 3
        for w in range(st["W"]):
            t_ = b * st["W"] + w
            ln = st["end"][b] - st["start"][b] + 1
            o = st["off_hist"][t_]
            if kind == 0 or (kind == 1 and w == 0):
                H[o:o + ln] = 100 + rng.integers(0, 10, ln).astype(np.uint64)
    t = Trio(cuda, ref, st)
    t.check_histogram(0.8)
    snap = t.check("check_histogram")
    assert np.any(snap["cond"] == 1) and np.any(snap["cond"] == 0)


@pytest.mark.parametrize("W", [1, 2])
def test_average_log_g_two_walkers(cuda, ref, W):
    """wl.cu:710-783 + :969-1031 with one or two walkers per window (the
    reference's FP64 atomics then add in an order-free way), flat and unflat
    windows, a finished sample."""
    rng = np.random.default_rng(11 + W)
    st = exact_state(5, 4, 1, 0.1, "v", 8, 3, 6, W, 0.25)
    roughen(st, rng)
    st["cond"][:] = rng.integers(0, 2, st["cond"].shape).astype(np.int8)
    st["cond_inter"][:] = [0, -1, 3]
    t = Trio(cuda, ref, st)
    t.average()
    t.check("average")


def test_reset_and_finished(cuda, ref):
    rng = np.random.default_rng(3)
    st = exact_state(4, 4, 0, 0.04, "i", 3, 4, 5, 3, 0.25)
    chain = sqrt_chain(12)
    st["factor"][:] = np.repeat(chain[rng.integers(0, 12, 20)], 3)
    st["cond"][:] = rng.integers(0, 2, 20).astype(np.int8)
    st["cond"][5:10] = 1
    t = Trio(cuda, ref, st)
    # a final ln f between two factors of the chain, so no factor sits at exp(beta)
    t.reset_finish(float(0.5 * (np.log(chain[6]) + np.log(chain[7]))))
    t.check("reset/finished")


def test_offsets_histogram_layout(cuda, ref):
    """wl.cu:615-652 gives the walker offsets the states here are built with."""
    torch = cuda
    import ctypes as C
    st = exact_state(6, 6, 0, 0.04, "i", 1, 3, 7, 3, 0.25)
    R, I, W = st["R"], st["I"], st["W"]
    lens = [int(sum(W * (st["end"][k * I + b] - st["start"][k * I + b] + 1) for b in range(I))) for k in range(R)]
    d_off = torch.zeros(R * I * W, dtype=torch.int32, device="cuda")
    d_s = torch.from_numpy(st["start"]).cuda()
    d_e = torch.from_numpy(st["end"]).cuda()
    d_l = torch.tensor(lens, dtype=torch.int32, device="cuda")
    v = lambda x: C.c_void_p(x.data_ptr())
    assert ref.refh_k_init_offsets_histogram(v(d_off), v(d_s), v(d_e), v(d_l), I, W, R * I * W) == 0
    assert np.array_equal(d_off.cpu().numpy(), st["off_hist"])


@pytest.mark.parametrize("X,Y,R,seed,prob", [(4, 4, 5, 1, 0.15), (6, 6, 3, 12345, 0.04), (7, 5, 4, -17, 0.5)])
@pytest.mark.parametrize("cls", ["i", "h", "v", "c"])
def test_init_interactions_and_energies(cuda, ref, X, Y, R, seed, prob, cls):
    """wl.cu:364-428 (disorder and error chains) and wl.cu:261-340 (energies)."""
    torch = cuda
    import ctypes as C
    import qec_pf_wang_landau_gb300 as wlg
    v = lambda x: C.c_void_p(x.data_ptr())
    N = X * Y
    d_ref = torch.zeros(R * 2 * N, dtype=torch.int8, device="cuda")
    d_eng = torch.zeros_like(d_ref)
    assert ref.refh_k_init_interactions(v(d_ref), X, Y, R, seed, C.c_float(prob), cls.encode()) == 0
    wlg.call("wlg_init_interactions", v(d_eng), N, R, seed, C.c_float(prob), None)
    wlg.call("wlg_apply_error_class", v(d_eng), X, Y, R, cls.encode(), None)
    J = d_ref.cpu().numpy()
    assert np.array_equal(J, d_eng.cpu().numpy())
    assert np.array_equal(J, O.init_interactions(X, Y, R, seed, prob, cls))
    wpi = 7
    nl = R * wpi
    rng = np.random.default_rng(abs(seed))
    lat = np.where(rng.random(nl * N) < 0.5, -1, 1).astype(np.int8)
    off = (np.arange(nl, dtype=np.int32) * N)
    d_lat, d_off, d_J = (torch.from_numpy(a).cuda() for a in (lat, off, J))
    for boundary in (0, 1):
        e_ref = torch.zeros(nl, dtype=torch.int32, device="cuda")
        e_eng = torch.zeros_like(e_ref)
        assert ref.refh_k_calc_energy(boundary, v(e_ref), v(d_lat), v(d_J), v(d_off), X, Y, nl, wpi) == 0
        wlg.call("wlg_calc_energy", boundary, v(e_eng), v(d_lat), v(d_J), v(d_off), X, Y, nl, wpi, None)
        a = e_ref.cpu().numpy()
        assert np.array_equal(a, e_eng.cpu().numpy())
        assert np.array_equal(a, O.calc_energy(boundary, lat, J, off, X, Y, nl, wpi))


@pytest.mark.parametrize("X,Y,boundary,cls", [(4, 4, 0, "i"), (6, 6, 0, "c"), (5, 7, 1, "v")])
def test_pre_run_one_walker_per_sample(cuda, ref, X, Y, boundary, cls):
    """wl.cu:473-560 (with store_lattice, :227-257) with one walker per sample:
    histogram, stored lattices and their flags, walker lattices, energies and
    RNG offsets after the walk."""
    torch = cuda
    import ctypes as C
    import qec_pf_wang_landau_gb300 as wlg
    v = lambda x: C.c_void_p(x.data_ptr())
    R, seed, n_iter, n_int = 24, 2024, 3000, 12
    N = X * Y
    J = O.init_interactions(X, Y, R, seed, 0.1, cls)
    lat = O.init_lattice(X, Y, R, seed, 1)
    off = np.arange(R, dtype=np.int32) * N
    E = O.calc_energy(boundary, lat, J, off, X, Y, R, 1)
    e_min, e_max = -2 * N, 2 * N
    _, _, _, len_int = O.interval_results(e_min, e_max, n_int, 1, 1.0)
    host = dict(E=E.copy(), flag=np.zeros(R * n_int, np.int32), lat=lat.copy(),
                found=np.zeros(R * n_int * N, np.int8), hist=np.zeros(R * (4 * N + 1), np.uint64),
                seed_off=np.zeros(R, np.uint64))
    dev = [{k: torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a.copy()).cuda()
            for k, a in host.items()} for _ in range(2)]
    d_J, d_off = torch.from_numpy(J).cuda(), torch.from_numpy(off).cuda()
    d = dev[0]
    assert ref.refh_k_pre_run(v(d["E"]), v(d["flag"]), v(d["lat"]), v(d["found"]), v(d["hist"]), v(d["seed_off"]),
                              v(d_J), v(d_off), e_min, e_max, n_iter, X, Y, seed, n_int, len_int, R, 1,
                              boundary) == 0
    d = dev[1]
    wlg.call("wlg_wang_landau_pre_run", v(d["E"]), v(d["flag"]), v(d["lat"]), v(d["found"]), v(d["hist"]),
             v(d["seed_off"]), v(d_J), v(d_off), e_min, e_max, n_iter, X, Y, seed, n_int, len_int, R, 1, boundary,
             None)
    p = O.ptr
    O.lib().orc_wang_landau_pre_run(p(host["E"]), p(host["flag"]), p(host["lat"]), p(host["found"]), p(host["hist"]),
                                    p(host["seed_off"]), p(J), p(off), e_min, e_max, n_iter, X, Y, seed, n_int,
                                    len_int, R, 1, boundary)
    torch.cuda.synchronize()
    for k, want in host.items():
        for name, dd in (("reference kernel", dev[0]), ("engine", dev[1])):
            got = dd[k].cpu().numpy()
            got = got.view(np.uint64) if want.dtype == np.uint64 else got
            assert np.array_equal(got, want), f"{k}: {name} vs oracle"
    assert np.all(host["seed_off"] >= n_iter) and host["flag"].sum() > R


def test_all_accept_step_replay(cuda, ref):
    """test_wang_landau.cu:162-488 re-expressed: 10 samples x 10 windows x 5
    walkers of random 4x4 lattices and couplings, every window the full range
    [-32, 32], every energy in the spectrum, log g = 0 and f = e: one step
    accepts every proposal (unless the uniform is exactly 1), so each walker's
    proposed site is flipped and H and log g gain 1 at the new energy."""
    torch = cuda
    R, I, W, X, Y, seed = 10, 10, 5, 4, 4, 42
    N, T = X * Y, R * I * W
    rng = np.random.default_rng(162)
    ln = 4 * N + 1
    st = dict(X=X, Y=Y, boundary=0, R=R, I=I, W=W, N=N,
              J=np.where(rng.random(R * 2 * N) < 0.5, -1, 1).astype(np.int8),
              spectrum=np.ones(R * ln, np.int8), off_spec=(np.arange(R, dtype=np.int32) * ln).astype(np.int32),
              start=np.full(R * I, -2 * N, np.int32), end=np.full(R * I, 2 * N, np.int32),
              off_hist=(np.arange(T, dtype=np.int32) * ln).astype(np.int32),
              lattice=np.where(rng.random(T * N) < 0.5, -1, 1).astype(np.int8),
              off_lat=(np.arange(T, dtype=np.int32) * N).astype(np.int32),
              H=np.zeros(T * ln, np.uint64), logG=np.zeros(T * ln), factor=np.full(T, np.e),
              off_iter=np.zeros(T, np.uint64), cond=np.zeros(R * I, np.int8), cond_inter=np.zeros(R, np.int32),
              perm=(np.arange(T) % W).astype(np.int32), found=np.zeros(T, np.int32), newE=np.zeros(T, np.int32))
    for boundary in (0, 1):
        st["boundary"] = boundary
        st["E"] = O.calc_energy(boundary, st["lattice"], st["J"], st["off_lat"], X, Y, T, I * W)
        t = Trio(torch, ref, st)
        t.wang_landau(1, seed)
        snap = t.check(f"boundary {boundary}")
        # the reference test's expectation, from the proposals' own draws
        u = np.array([O.uniforms(seed + q // (I * W), q % (I * W), 0, 2) for q in range(T)])
        site = np.trunc(u[:, 0].astype(np.float64) * (N - 1 + 0.999999)).astype(np.int64)
        lat = st["lattice"].copy()
        for q in range(T):
            if u[q, 1] < 1.0:
                lat[q * N + site[q]] *= -1
        assert np.array_equal(snap["lattice"], lat)
        E2 = O.calc_energy(boundary, lat, st["J"], st["off_lat"], X, Y, T, I * W)
        assert np.array_equal(snap["E"], E2)
        H = np.zeros(T * ln, np.uint64)
        H[st["off_hist"] + E2 + 2 * N] += 1
        assert np.array_equal(snap["H"], H)
        assert np.array_equal(snap["logG"], H.astype(np.float64))


def test_full_main_run_equals_reference_kernels(cuda, ref):
    """The reference's main loop (mainrun.cu:235-383 on its kernels, exchange
    counter never advancing, Q14) from the pre-run outputs, against this
    engine's persistent batched main run (exchange_mode 0) from the same
    pre-run: every window's walker-0 log g equal bit for bit, 6x6 periodic,
    the four classes, two walkers per window."""
    import qec_pf_wang_landau_gb300 as wlg
    X, Y, seed, R, pre_w, pre_i, pre_n, I, W = 6, 6, 12345, 3, 128, 32, 1000, 10, 2
    ctx = wlg.Context(0)
    for cls in "ivhc":
        pre = prerun_outputs(X, Y, 0, 0.04, cls, seed, R, pre_w, pre_i, pre_n)
        N = X * Y
        for k in range(R):
            cnt = O.exact_counts(pre["J"][k * 2 * N:(k + 1) * 2 * N], X, Y, 0)
            assert np.array_equal(pre["seen"][k * (4 * N + 1):(k + 1) * (4 * N + 1)] != 0, cnt != 0)
        lat = pre["found_lat"].copy()
        for q in range(R * pre_i):
            if not pre["found_flag"][q]:
                lat[q * N:(q + 1) * N] = 0
        out = O.reference_mainrun(X, Y, 0, seed, R, pre_i, pre["seen"], pre["J"], lat, pre["found_energy"], I, W,
                                  0.25, 0.8, 1e-3, 1000, 20)
        assert out["status"] == 0
        probs = [wlg.problem(X, Y, prob=0.04, error_class=cls, seed=seed, sample=k, pre_walkers=pre_w,
                             pre_intervals=pre_i, pre_iterations=pre_n, intervals=I, walkers_per_interval=W,
                             exchange_mode=0, global_parity=1) for k in range(R)]
        mine = ctx.solve_raw(probs)
        for k, (r, s, e, wins) in enumerate(mine):
            assert r.status == 0
            assert np.array_equal(s, out["start"][k * I:(k + 1) * I]) and np.array_equal(e, out["end"][k * I:(k + 1) * I])
            for b in range(I):
                assert np.array_equal(wins[b], out["windows"][k * I + b]), (cls, k, b)


@pytest.mark.parametrize("X,Y,boundary,cls", [(6, 6, 0, "c"), (5, 6, 1, "h")])
def test_batched_exchange_every_iteration_equals_reference_kernels(cuda, ref, X, Y, boundary, cls):
    """The reference's main loop at -c 1 exchanges every outer iteration
    (its counter stays 1, mainrun.cu:241, :346).  From the same pre-run, its
    kernels and this engine's persistent batched main run (exchange mode 0,
    every iteration, the reference's global parity) give equal walker-0 log g
    in every window after 25 outer iterations, bit for bit; ln f never reaches
    its final value in that span (2^-25 > 1e-9), so no window finishes and the
    reference's finished-window walk (Q5) is not entered; two walkers per window
    keep its averaging order-free.  Without exchange the result differs."""
    import qec_pf_wang_landau_gb300 as wlg
    seed, R, pre_w, pre_i, pre_n, I, W, cap = 4321, 3, 64, 16, 4000, 8, 2, 25
    N = X * Y
    pre = prerun_outputs(X, Y, boundary, 0.1, cls, seed, R, pre_w, pre_i, pre_n)
    for k in range(R):
        cnt = O.exact_counts(pre["J"][k * 2 * N:(k + 1) * 2 * N], X, Y, boundary)
        assert np.array_equal(pre["seen"][k * (4 * N + 1):(k + 1) * (4 * N + 1)] != 0, cnt != 0)
    lat = pre["found_lat"].copy()
    for q in range(R * pre_i):
        if not pre["found_flag"][q]:
            lat[q * N:(q + 1) * N] = 0
    out = O.reference_mainrun(X, Y, boundary, seed, R, pre_i, pre["seen"], pre["J"], lat, pre["found_energy"], I, W,
                              0.3, 0.8, 1e-9, 500, 1, max_outer=cap)
    assert out["status"] == 3 and out["outer"] == cap

    def mine(xc):
        probs = [wlg.problem(X, Y, boundary=boundary, prob=0.1, error_class=cls, seed=seed, sample=k,
                             pre_walkers=pre_w, pre_intervals=pre_i, pre_iterations=pre_n, intervals=I,
                             walkers_per_interval=W, overlap=0.3, beta=1e-9, iterations=500, exchange_every=xc,
                             exchange_mode=0, global_parity=1, max_outer=cap) for k in range(R)]
        return wlg.Context(0).solve_raw(probs)
    with_x, without_x = mine(1), mine(2)
    differs = False
    for k in range(R):
        r, s, e, wins = with_x[k]
        assert r.status == 7 and r.outer_iterations == cap  # WLG_ERR_TIMEOUT at the cap
        assert np.array_equal(s, out["start"][k * I:(k + 1) * I]) and np.array_equal(e, out["end"][k * I:(k + 1) * I])
        for b in range(I):
            assert np.array_equal(wins[b], out["windows"][k * I + b]), (k, b)
            differs |= not np.array_equal(without_x[k][3][b], wins[b])
    assert differs
