"""GPU parity of the operator layer (reference layout) against the oracle.

Integer outputs (couplings, lattices, energies, histograms, flags, RNG
offsets, exchange decisions) must be bit-exact; log g too, because both
sides perform the same FP64 operations in the same order.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import oracle as O
from tests.helpers import (Dev, assert_state_equal, copy_state, mainrun_state, o_average, o_check_histogram,
                           o_exchange, o_reset_finish, o_wang_landau, prerun_outputs)

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe(cuda):
    sys.path.insert(0, os.path.join(HERE, "csrc"))
    import build_probe
    L = C.CDLL(build_probe.build())
    for n in ("probe_curand_uniform", "probe_exp_log", "probe_sqrt_chain"):
        getattr(L, n).restype = C.c_int
    L.probe_sqrt_chain.argtypes = [C.c_double, C.c_int, C.c_void_p, C.c_void_p]
    return L


def _dptr(t):
    return C.c_void_p(t.data_ptr())


TRIPLES = [(0, 0, 0), (1, 0, 0), (12345, 0, 5), (12345, 3, 0), (12345, 3, 1), (12345, 3, 2), (12345, 3, 3),
           (12345, 29, 1001), (2 ** 32 + 7, 2, 77), ((-5) % 2 ** 64, 1, 13), (4294967291, 127, 2 ** 33 + 3),
           (987654321, 2 ** 40 + 5, 3), (42, 0, 123456789), (7, 1, 31)]


def test_philox_streams_match_curand(cuda, probe):
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    n_draws = 37
    seeds = torch.tensor(np.array([t[0] for t in TRIPLES], np.uint64).view(np.int64)).cuda()
    subs = torch.tensor(np.array([t[1] for t in TRIPLES], np.uint64).view(np.int64)).cuda()
    offs = torch.tensor(np.array([t[2] for t in TRIPLES], np.uint64).view(np.int64)).cuda()
    ref = torch.zeros(len(TRIPLES) * n_draws, dtype=torch.float32, device="cuda")
    assert probe.probe_curand_uniform(_dptr(seeds), _dptr(subs), _dptr(offs), len(TRIPLES), n_draws, _dptr(ref)) == 0
    ref = ref.cpu().numpy().reshape(len(TRIPLES), n_draws)
    mine = torch.zeros(n_draws, dtype=torch.float32, device="cuda")
    for q, (k, s, o) in enumerate(TRIPLES):
        wlg.call("wlg_uniforms", k, s, o, n_draws, _dptr(mine), None)
        torch.cuda.synchronize()
        got = mine.cpu().numpy()
        host = O.uniforms(k, s, o, n_draws)
        assert np.array_equal(got.view(np.uint32), ref[q].view(np.uint32)), f"engine vs cuRAND, triple {q}"
        assert np.array_equal(host.view(np.uint32), ref[q].view(np.uint32)), f"oracle vs cuRAND, triple {q}"


def test_device_log_of_factor_chain_matches_host(cuda, probe):
    """ln f of every modification factor e, e^(1/2), e^(1/4), ... is bit-identical on host and device."""
    torch = cuda
    n = 60
    f = torch.zeros(n, dtype=torch.float64, device="cuda")
    lf = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert probe.probe_sqrt_chain(np.e, n, _dptr(f), _dptr(lf)) == 0
    hf = np.zeros(n)
    hlf = np.zeros(n)
    O.lib().orc_sqrt_chain(np.e, n, O.ptr(hf), O.ptr(hlf))
    assert np.array_equal(f.cpu().numpy(), hf)
    assert np.array_equal(lf.cpu().numpy(), hlf)


def test_prerun_acceptance_exp_decisions_match(cuda, probe):
    """exp(H_old - H_new) of integer count differences: every float uniform
    compares the same way against the device and host values."""
    torch = cuda
    x = np.arange(-1100, 1101, dtype=np.float64)
    dx = torch.from_numpy(x).cuda()
    de = torch.zeros_like(dx)
    dl = torch.zeros_like(dx)
    assert probe.probe_exp_log(_dptr(dx), _dptr(de), _dptr(dl), len(x)) == 0
    he = np.zeros_like(x)
    hl = np.zeros_like(x)
    O.lib().orc_exp_log(O.ptr(np.ascontiguousarray(x)), O.ptr(he), O.ptr(hl), len(x))
    ge = de.cpu().numpy()
    u_min = 2.0 ** -33  # the smallest uniform a draw can give
    n_diff = 0
    for a, b in zip(ge, he):
        lo, hi = min(a, b), max(a, b)
        if lo == hi or hi < u_min:
            continue
        n_diff += 1
        # no reachable float uniform u may satisfy lo <= u < hi
        if lo > 1.0:
            continue
        f = np.float32(max(lo, u_min))
        f = f if float(f) >= lo else np.nextafter(f, np.float32(np.inf))
        assert not (lo <= float(f) < hi), (a, b)
    assert n_diff < len(x) // 10


@pytest.mark.parametrize("X,Y,R,seed,prob", [(4, 4, 3, 1, 0.15), (6, 6, 5, 12345, 0.04), (7, 5, 4, -17, 0.5),
                                             (24, 24, 2, 99, 0.1), (3, 9, 6, 2 ** 31 - 3, 0.3)])
@pytest.mark.parametrize("cls", ["i", "h", "v", "c"])
def test_init_interactions(cuda, X, Y, R, seed, prob, cls):
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    d = torch.zeros(R * 2 * X * Y, dtype=torch.int8, device="cuda")
    wlg.call("wlg_init_interactions", _dptr(d), X * Y, R, seed, C.c_float(prob), None)
    wlg.call("wlg_apply_error_class", _dptr(d), X, Y, R, cls.encode(), None)
    ref = O.init_interactions(X, Y, R, seed, prob, cls)
    assert np.array_equal(d.cpu().numpy(), ref)


@pytest.mark.parametrize("X,Y,nl,seed,wpi", [(4, 4, 10, 5, 5), (6, 6, 12, 12345, 4), (5, 7, 9, -3, 3),
                                             (24, 24, 4, 1, 2)])
def test_init_lattice(cuda, X, Y, nl, seed, wpi):
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    d = torch.zeros(nl * X * Y, dtype=torch.int8, device="cuda")
    wlg.call("wlg_init_lattice", _dptr(d), X, Y, nl, seed, wpi, None)
    assert np.array_equal(d.cpu().numpy(), O.init_lattice(X, Y, nl, seed, wpi))


@pytest.mark.parametrize("boundary", [0, 1])
@pytest.mark.parametrize("X,Y", [(4, 4), (6, 6), (5, 3), (16, 16), (24, 24)])
def test_calc_energy(cuda, boundary, X, Y):
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    rng = np.random.default_rng(X * 100 + Y + boundary)
    R, wpi = 3, 4
    nl = R * wpi
    lat = rng.choice(np.array([-1, 1], np.int8), nl * X * Y)
    J = rng.choice(np.array([-1, 1], np.int8), R * 2 * X * Y)
    off = (np.arange(nl) * X * Y).astype(np.int32)
    dl, dJ, do = (torch.from_numpy(a).cuda() for a in (lat, J, off))
    dE = torch.zeros(nl, dtype=torch.int32, device="cuda")
    wlg.call("wlg_calc_energy", boundary, _dptr(dE), _dptr(dl), _dptr(dJ), _dptr(do), X, Y, nl, wpi, None)
    assert np.array_equal(dE.cpu().numpy(), O.calc_energy(boundary, lat, J, off, X, Y, nl, wpi))


def test_calc_energy_known_answers(cuda):
    """test_calc_energy.cu: -6 periodic / -4 open for the literal 4x4 case; all-up lattices."""
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    lat = np.array([1, 1, -1, 1, -1, -1, 1, -1, 1, -1, 1, -1, -1, -1, -1, -1], np.int8)
    J = np.array([1, -1, 1, 1, 1, 1, 1, 1, -1, 1, 1, -1, 1, 1, 1, 1, 1, 1, -1, 1, 1, 1, 1, 1, -1, 1, 1, 1, 1, 1, 1,
                  1], np.int8)
    dlat, dJ = torch.from_numpy(lat).cuda(), torch.from_numpy(J).cuda()  # keep the buffers alive
    doff = torch.zeros(1, dtype=torch.int32, device="cuda")
    for boundary, want in ((0, -6), (1, -4)):
        dE = torch.zeros(1, dtype=torch.int32, device="cuda")
        wlg.call("wlg_calc_energy", boundary, _dptr(dE), _dptr(dlat), _dptr(dJ), _dptr(doff), 4, 4, 1, 1, None)
        assert int(dE.item()) == want
    ones = torch.ones(10 * 16, dtype=torch.int8, device="cuda")
    Jones = torch.ones(2 * 32, dtype=torch.int8, device="cuda")
    off = torch.arange(10, dtype=torch.int32, device="cuda") * 16
    for boundary, want in ((0, -32), (1, -32 + 8)):
        dE = torch.zeros(10, dtype=torch.int32, device="cuda")
        wlg.call("wlg_calc_energy", boundary, _dptr(dE), _dptr(ones), _dptr(Jones), _dptr(off), 4, 4, 10, 5, None)
        assert (dE.cpu().numpy() == want).all()


@pytest.mark.parametrize("X,Y,boundary,R,wpi,n_int,n_iter,seed,prob", [
    (4, 4, 0, 2, 32, 8, 500, 12345, 0.04),
    (4, 4, 1, 2, 16, 5, 300, 7, 0.0),
    (6, 6, 0, 3, 128, 32, 200, 12345, 0.04),
    (5, 7, 1, 2, 40, 9, 150, -11, 0.2),
])
def test_prerun_walk(cuda, X, Y, boundary, R, wpi, n_int, n_iter, seed, prob):
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    N = X * Y
    J = O.init_interactions(X, Y, R, seed, prob, "v")
    T = R * wpi
    lat = O.init_lattice(X, Y, T, seed, wpi)
    off = (np.arange(T) * N).astype(np.int32)
    E = O.calc_energy(boundary, lat, J, off, X, Y, T, wpi)
    s, e, _, len_int = O.interval_results(-2 * N, 2 * N, n_int, 1, 1.0)
    L = 4 * N + 1
    H = np.zeros(R * L, np.uint64)
    flags = np.zeros(R * n_int, np.int32)
    flat = np.zeros(R * n_int * N, np.int8)
    so = np.zeros(T, np.uint64)
    dev = {k: torch.from_numpy(v.view(np.int64) if v.dtype == np.uint64 else v.copy()).cuda()
           for k, v in dict(E=E, flags=flags, lat=lat, flat=flat, H=H, so=so, J=J, off=off).items()}
    wlg.call("wlg_wang_landau_pre_run", _dptr(dev["E"]), _dptr(dev["flags"]), _dptr(dev["lat"]), _dptr(dev["flat"]),
             _dptr(dev["H"]), _dptr(dev["so"]), _dptr(dev["J"]), _dptr(dev["off"]), -2 * N, 2 * N, n_iter, X, Y,
             seed, n_int, len_int, T, wpi, boundary, None)
    p = O.ptr
    O.lib().orc_wang_landau_pre_run(p(E), p(flags), p(lat), p(flat), p(H), p(so), p(J), p(off), -2 * N, 2 * N, n_iter,
                                    X, Y, seed, n_int, len_int, T, wpi, boundary)
    torch.cuda.synchronize()
    assert np.array_equal(dev["E"].cpu().numpy(), E)
    assert np.array_equal(dev["lat"].cpu().numpy(), lat)
    assert np.array_equal(dev["H"].cpu().numpy().view(np.uint64), H)
    assert np.array_equal(dev["flags"].cpu().numpy(), flags)
    assert np.array_equal(dev["flat"].cpu().numpy(), flat)
    assert np.array_equal(dev["so"].cpu().numpy().view(np.uint64), so)
    assert (so == 2 * n_iter).all()


CASES = [
    # X, Y, boundary, R, I, W, overlap, cls, seed, prob, n_iter, iters, exchange_every
    (4, 4, 0, 2, 4, 3, 0.25, "i", 12345, 0.04, 200, 40, 1),
    (4, 4, 1, 2, 3, 4, 0.3, "c", 99, 0.1, 150, 30, 2),
    (6, 6, 0, 3, 10, 3, 0.25, "v", 12345, 0.04, 300, 25, 3),
    (5, 4, 1, 2, 5, 2, 0.5, "h", -21, 0.2, 100, 30, 1),
]


@pytest.mark.parametrize("X,Y,boundary,R,I,W,overlap,cls,seed,prob,n_iter,iters,xc", CASES)
def test_mainrun_operators_step_by_step(cuda, X, Y, boundary, R, I, W, overlap, cls, seed, prob, n_iter, iters, xc):
    """The reference's outer loop (mainrun.cu:243-374) driven through the
    operators on GPU and on the oracle; every array equal after every step."""
    torch = cuda
    pre = prerun_outputs(X, Y, boundary, prob, cls, seed, R, 32, 12, 2000)
    st = mainrun_state(pre, I, W, overlap)
    dev = Dev(torch, copy_state(st))
    alpha, beta = 0.8, 0.05
    for it in range(iters):
        n_new = o_wang_landau(st, n_iter, seed)
        dev.wang_landau(n_iter, seed)
        assert_state_equal(dev.snapshot(), st, f"iter {it} wang_landau")
        assert n_new == 0
        o_check_histogram(st, alpha)
        dev.check_histogram(alpha)
        o_average(st)
        dev.average()
        o_reset_finish(st, beta)
        dev.reset_finish(beta)
        assert_state_equal(dev.snapshot(), st, f"iter {it} flatness")
        if (it + 1) % xc == 0:
            for even in (1, 0):
                o_exchange(st, even, seed, global_parity=it % 2)
                dev.exchange(even, seed, global_parity=it % 2)
            assert_state_equal(dev.snapshot(), st, f"iter {it} exchange")
    # the run made progress: some windows went flat at least once
    assert (st["factor"] < np.e).any()


def test_new_energy_flags(cuda):
    torch = cuda
    pre = prerun_outputs(4, 4, 0, 0.04, "i", 3, 2, 32, 8, 2000)
    st = mainrun_state(pre, 3, 2, 0.25)
    # punch a hole into sample 1's spectrum at a reachable energy
    k = 1
    lo = st["off_spec"][k]
    hole = lo + 2 * 4 if st["spectrum"][lo + 8] == 1 else lo + 4 * 3
    st["spectrum"][hole] = 0
    dev = Dev(torch, copy_state(st))
    for _ in range(20):
        o_wang_landau(st, 500, 3)
        dev.wang_landau(500, 3)
    assert_state_equal(dev.snapshot(), st, "new energy")
    assert (st["found"][:6] == 0).all()
    assert (st["found"][6:] != 0).any()


def test_check_histogram_reference_vector(cuda):
    """test_check_histogram.cu:23-126 on the GPU."""
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    H = np.full(80, 10, np.uint64)
    H[0] = 1
    start = np.array([-2, -1, 0, -4, -2, 0, -2, -1, 0], np.int32)
    end = np.array([-1, 0, 2, -2, 0, 2, -2, -1, 1], np.int32)
    cond_inter = np.array([1, 1, 1], np.int32)
    off_hist = np.array([0, 2, 4, 6, 8, 10, 12, 14] + [16 + 3 * q for q in range(16)] + [64 + q for q in range(8)]
                        + [72, 74, 76, 78], np.int32)
    cond = np.array([0, 0, 0, 0, 0, 0, 0, 0, 1], np.int8)
    off_spec = np.array([0, 7, 16], np.int32)
    spec = np.ones(20, np.int8)
    factor = np.full(36, np.e)
    d = {k: torch.from_numpy(v.view(np.int64) if v.dtype == np.uint64 else v.copy()).cuda()
         for k, v in dict(H=H, factor=factor, cond=cond, off_hist=off_hist, end=end, start=start, spec=spec,
                          off_spec=off_spec, ci=cond_inter).items()}
    wlg.call("wlg_check_histogram", _dptr(d["H"]), _dptr(d["factor"]), _dptr(d["cond"]), _dptr(d["off_hist"]),
             _dptr(d["end"]), _dptr(d["start"]), _dptr(d["spec"]), _dptr(d["off_spec"]), _dptr(d["ci"]), 0.8, 36, 12,
             3, None)
    torch.cuda.synchronize()
    want_H = np.zeros(80, np.uint64)
    want_H[:8] = 10
    want_H[72:] = 10
    want_H[0] = 1
    assert np.array_equal(d["H"].cpu().numpy().view(np.uint64), want_H)
    assert d["cond"].cpu().numpy().tolist() == [0, 1, 1, 1, 1, 1, 1, 1, 1]
    want_f = np.full(36, np.sqrt(np.e))
    want_f[:4] = np.e
    want_f[32:] = np.e
    assert np.allclose(d["factor"].cpu().numpy(), want_f, rtol=1e-15, atol=0)


def test_replica_exchange_flat_log_g_swaps_by_permutation(cuda):
    """test_replica_exchange.cu:36-158: with flat log g every admissible pair swaps."""
    torch = cuda
    R, I, W = 3, 10, 5
    T = R * I * W
    start = np.zeros(R * I, np.int32)
    end = np.zeros(R * I, np.int32)
    E = np.zeros(T, np.int32)
    off_hist = np.zeros(T, np.int32)
    off_lat = np.zeros(T, np.int32)
    acc = 0
    for b in range(R * I):
        bl, k = b % I, b // I
        start[b], end[b] = bl + k, bl + k + 4
        for w in range(W):
            t = b * W + w
            E[t] = bl + k + 2
            off_hist[t] = acc
            acc += 5
            off_lat[t] = t * 9
    st = dict(R=R, I=I, W=W, start=start, end=end, E=E, off_hist=off_hist, off_lat=off_lat,
              logG=np.ones(acc), perm=(np.arange(T) % W).astype(np.int32), off_iter=np.zeros(T, np.uint64),
              cond_inter=np.ones(R, np.int32))
    ref = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
    o_exchange(ref, 1, 42, global_parity=1)
    import qec_pf_wang_landau_gb300 as wlg
    d = {k: torch.from_numpy(v.view(np.int64) if v.dtype == np.uint64 else v.copy()).cuda() for k, v in st.items()
         if isinstance(v, np.ndarray)}
    wlg.call("wlg_replica_exchange", _dptr(d["off_lat"]), _dptr(d["E"]), _dptr(d["perm"]), _dptr(d["off_iter"]),
             _dptr(d["start"]), _dptr(d["end"]), _dptr(d["off_hist"]), _dptr(d["cond_inter"]), _dptr(d["logG"]), 1, 42,
             I, I * W, R * I, 1, None)
    torch.cuda.synchronize()
    got_off = d["off_lat"].cpu().numpy()
    perm = d["perm"].cpu().numpy()
    assert np.array_equal(got_off, ref["off_lat"])
    assert np.array_equal(perm, ref["perm"])
    assert np.array_equal(d["off_iter"].cpu().numpy().view(np.uint64), ref["off_iter"])
    for b in range(R * I):
        if b % I == I - 1 or b % 2:
            continue
        assert sorted(perm[b * W:(b + 1) * W].tolist()) == list(range(W))
        for w in range(W):
            t = b * W + w
            o = (b + 1) * W + perm[t]
            assert got_off[t] == off_lat[o] and got_off[o] == off_lat[t]


def test_fast_exp_within_bound_used_by_acceptance(cuda, probe):
    """The engine's FP32 acceptance test assumes |__expf(x) / exp(x) - 1| <= (2 + 1.2|x|) 2^-23
    for normal results; checked on a dense grid of [-87, 0]."""
    torch = cuda
    x = np.concatenate([np.linspace(-87.0, 0.0, 2_000_001, dtype=np.float32),
                        -np.logspace(-30, 1, 100_001).astype(np.float32)])
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros_like(dx)
    probe.probe_fast_exp.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    assert probe.probe_fast_exp(_dptr(dx), _dptr(dy), len(x)) == 0
    y = dy.cpu().numpy().astype(np.float64)
    ex = np.exp(x.astype(np.float64))
    ok = ex > 1.2e-38
    rel = np.abs(y[ok] / ex[ok] - 1.0)
    bound = (2.0 + 1.2 * np.abs(x[ok].astype(np.float64))) * 2.0 ** -23
    assert (rel <= bound).all(), float((rel / bound).max())


def test_split_shadow_error_bound(cuda, probe):
    """The sweep's shadow of g - base (written on every change of bin), formed
    from float splits of the doubles, is within 2^-23 |g - base| +
    2^-44 (g + base) of the exact difference (values below 2^-126 count as 0)."""
    from fractions import Fraction
    torch = cuda
    rng = np.random.default_rng(7)
    n = 20000
    base = 10.0 ** rng.uniform(-8, 5, n)
    r = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-16, 0.5, n)
    g = np.abs(base * (1.0 + r))
    g[:200] = base[:200]                                              # equal
    g[200:400] = base[200:400] * 2.0 ** rng.integers(-70, 71, 200)    # binades apart
    g[400:450] = 0.0
    base[450:500] = 0.0
    g[500:550], base[500:550] = 1e-40, 3e-39                          # below 2^-126
    g[550:600] = 1e30
    dg, db = torch.from_numpy(g).cuda(), torch.from_numpy(base).cuda()
    out = torch.zeros(n, dtype=torch.float32, device="cuda")
    probe.probe_shadow.argtypes = [C.c_void_p] * 3 + [C.c_int]
    assert probe.probe_shadow(_dptr(dg), _dptr(db), _dptr(out), n) == 0
    out = out.cpu().numpy()
    tiny = Fraction(1, 2 ** 126)
    for q in range(n):
        gq = Fraction(float(g[q])) if g[q] >= 2.0 ** -126 else Fraction(0)
        bq = Fraction(float(base[q])) if base[q] >= 2.0 ** -126 else Fraction(0)
        exact = gq - bq
        bound = abs(exact) / 2 ** 23 + (gq + bq) / 2 ** 44 + 2 * tiny
        assert abs(Fraction(float(out[q])) - exact) <= bound, (g[q], base[q], out[q])


def test_fast_log_error_within_engine_bound(cuda, probe):
    """The sweep decides log u < d with u's __logf; its error bound holds for
    every float u in [2^-33, 1] (exhaustive, against FP64 log)."""
    torch = cuda
    probe.probe_log_bound.restype = C.c_float
    bound = probe.probe_log_bound()
    mx = torch.zeros(1, dtype=torch.int32, device="cuda")
    probe.probe_logf_maxerr.argtypes = [C.c_uint, C.c_uint, C.c_void_p]
    lo = int(np.float32(2.0 ** -33).view(np.uint32))
    hi = int(np.float32(1.0).view(np.uint32))
    assert probe.probe_logf_maxerr(lo, hi, _dptr(mx)) == 0
    worst = float(mx.cpu().numpy().view(np.float32)[0])
    assert 0.0 < worst <= bound, (worst, bound)


def test_fast_decision_never_contradicts_exact_rule(cuda, probe):
    """decide(): whenever it reports the answer as known it equals the
    reference's u < min(1, exp(d)), for estimates df within eps of d, most of
    all next to the boundary log u = d."""
    torch = cuda
    rng = np.random.default_rng(11)
    n = 2_000_000
    x = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    x[:1000] = 0xFFFFFFFF - np.arange(1000, dtype=np.uint32)  # u = 1
    u = ((x.astype(np.float64) + 0.5) * 2.0 ** -32).astype(np.float32).astype(np.float64)
    d = rng.uniform(-12.0, 1.0, n)
    near = rng.random(n) < 0.5
    d[near] = np.log(u[near]) + rng.choice([-1.0, 1.0], near.sum()) * 10.0 ** rng.uniform(-9, -3, near.sum())
    eps = (10.0 ** rng.uniform(-9, -4, n)).astype(np.float32)
    noise = rng.uniform(-0.5, 0.5, n) * eps
    df = (d + noise).astype(np.float32)
    eps = (eps.astype(np.float64) + np.abs(df.astype(np.float64) - (d + noise))).astype(np.float32) * np.float32(1.0001)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tx, td, tdf, te = dev(x.view(np.int32)), dev(d), dev(df), dev(eps)
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    probe.probe_decide.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p]
    assert probe.probe_decide(_dptr(tx), _dptr(td), _dptr(tdf), _dptr(te), n, _dptr(out)) == 0
    o = out.cpu().numpy()
    assert (o >= 0).all(), int((o < 0).sum())
    assert (o[~near] == 0).mean() < 1e-3   # away from the boundary almost everything is settled in FP32


def test_device_exp_of_nonnegative_is_at_least_one(cuda, probe):
    """min(1, exp(d)) == 1 for every d >= 0 (the acceptance shortcut for d >= 0)."""
    torch = cuda
    x = np.concatenate([[0.0], np.logspace(-320, 2, 20001)])
    dx = torch.from_numpy(x).cuda()
    de = torch.zeros_like(dx)
    dl = torch.zeros_like(dx)
    assert probe.probe_exp_log(_dptr(dx), _dptr(de), _dptr(dl), len(x)) == 0
    assert (de.cpu().numpy() >= 1.0).all()


@pytest.mark.parametrize("case", ["none", "all", "some"])
def test_reset_cond_reference_cases(cuda, case):
    """test_reset_d_cond.cu:22/50/79: 2 samples x 10 windows x 20 walkers,
    beta 1e-10; factors at exp(beta) keep every flag, factors 1e-3 above it
    reset every flag, and raising only the last sample's factors resets only
    its windows."""
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    beta, R, I, W = 1e-10, 2, 10, 20
    factor = np.full(R * I * W, np.exp(beta))
    if case == "all":
        factor += 1e-3
    if case == "some":
        factor[(R - 1) * I * W:] += 1e-3
    cond = torch.ones(R * I, dtype=torch.int8, device="cuda")
    f = torch.from_numpy(factor).cuda()
    wlg.call("wlg_reset_cond", _dptr(cond), _dptr(f), R * I, C.c_double(beta), W, None)
    torch.cuda.synchronize()
    got = cond.cpu().numpy()
    want = np.ones(R * I, np.int8)
    if case == "all":
        want[:] = 0
    if case == "some":
        want[(R - 1) * I:] = 0
    assert np.array_equal(got, want)


@pytest.mark.parametrize("case", ["all_finished", "last_not_finished", "none_finished"])
def test_check_finished_reference_cases(cuda, case):
    """test_check_interactions.cu:17/58/105: 100 samples x 20 windows; -1
    marks a sample whose windows are all flat."""
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    R, I = 100, 20
    cond = np.ones(R * I, np.int8) if case != "none_finished" else np.zeros(R * I, np.int8)
    if case == "last_not_finished":
        cond[-1] = 0
    d_cond = torch.from_numpy(cond).cuda()
    out = torch.zeros(R, dtype=torch.int32, device="cuda")
    wlg.call("wlg_check_finished", _dptr(out), _dptr(d_cond), I, R, None)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    if case == "all_finished":
        assert (got == -1).all()
    elif case == "last_not_finished":
        assert (got[:-1] == -1).all() and got[-1] == I - 1
    else:
        assert (got == 0).all()


def test_measure_peaks(cuda):
    """wlg_measure_peaks: every rate positive and finite, the SM count the
    device's, shared-memory bandwidth above a plain HBM copy's order of
    magnitude and Philox well above a draw per flip of the engine; a null
    output is rejected and the current device is left as it was."""
    torch = cuda
    import qec_pf_wang_landau_gb300 as wlg
    before = torch.cuda.current_device()
    pk = wlg.measure_peaks(0)
    assert torch.cuda.current_device() == before
    assert pk["sm_count"] == torch.cuda.get_device_properties(0).multi_processor_count
    for k in ("smem_gbs", "philox_draws_per_s", "exp_f64_per_s", "log_f64_per_s"):
        assert np.isfinite(pk[k]) and pk[k] > 0, k
    assert pk["smem_gbs"] > 1000.0 and pk["philox_draws_per_s"] > 1e10
    assert wlg.lib().wlg_measure_peaks(0, None) == 1  # WLG_ERR_INVALID
