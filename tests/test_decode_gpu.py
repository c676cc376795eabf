"""Given disorder on the GPU: wlg_solve_couplings and
wlg_server_submit_couplings.

Couplings equal to the ones the pre-run draws must give the drawn runs'
results bit for bit (only the disorder stream is replaced); decoding a
syndrome through the server must give the exact class probabilities of the
syndrome's pattern (oracle transfer matrix) to Wang-Landau accuracy."""
import numpy as np
import pytest

import oracle as O
from test_server_gpu import as_tuple, request, same

pytestmark = pytest.mark.gpu

CASES = [  # X, Y, boundary, prob, cls, seed, sample
    (4, 4, 0, 0.06, "i", 12345, 0),
    (5, 4, 1, 0.15, "h", 99, 2),
    (6, 6, 0, 0.04, "c", 7, 1),
    (7, 5, 1, 0.10, "v", 31337, 3),
]


def problem(wlg, X, Y, boundary, prob, cls, seed, sample):
    return wlg.problem(X, Y, boundary=boundary, prob=prob, error_class=cls, seed=seed, sample=sample,
                       pre_walkers=64, pre_intervals=16, pre_iterations=2000, intervals=6, walkers_per_interval=3,
                       overlap=0.25, alpha=0.8, beta=1e-3, iterations=800, exchange_every=2)


def drawn_i(X, Y, seed, prob, sample):
    """Class-'i' couplings of (seed, sample) as the pre-run draws them."""
    return O.init_interactions(X, Y, sample + 1, seed, prob, "i")[sample * 2 * X * Y:(sample + 1) * 2 * X * Y]


def test_given_drawn_couplings_reproduce_solve(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    probs = [problem(wlg, *c) for c in CASES]
    J = [drawn_i(c[0], c[1], c[5], c[3], c[6]) for c in CASES]
    ctx = wlg.Context(0)
    a = ctx.solve(probs)
    b = ctx.solve(probs, couplings=J)
    for (ra, Ea, Ga), (rb, Eb, Gb) in zip(a, b):
        assert (ra.status, ra.outer_iterations, ra.flips, ra.pre_flips) == \
            (rb.status, rb.outer_iterations, rb.flips, rb.pre_flips)
        assert np.array_equal(Ea, Eb) and np.array_equal(Ga, Gb)
    assert any(r.status == 0 for r, _, _ in a)


def test_given_couplings_change_only_the_disorder(cuda):
    """A pattern other than the drawn one (here: the drawn one of another
    sample) gives that sample's log g curve family, not this one's: the
    energies reached follow the couplings."""
    import qec_pf_wang_landau_gb300 as wlg
    X, Y = 4, 4
    p = problem(wlg, X, Y, 0, 0.1, "i", 5, 0)
    J1 = drawn_i(X, Y, 5, 0.1, 1)
    (r, E, G), = wlg.Context(0).solve([p], couplings=[J1])
    assert r.status == 0
    cnt = O.exact_counts(J1, X, Y, 0)
    assert set(E.tolist()) == set((np.nonzero(cnt)[0] - 2 * X * Y).tolist())
    err = G - np.log(cnt[E + 2 * X * Y])
    assert np.sqrt(np.mean(err ** 2)) < 0.3


def test_invalid_couplings_rejected(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    p = problem(wlg, 4, 4, 0, 0.1, "i", 5, 0)
    bad = np.ones(32, np.int8)
    bad[7] = 0
    with pytest.raises(wlg.WlgError) as e:
        wlg.Context(0).solve([p], couplings=[bad])
    assert e.value.status == 1
    with wlg.Server(0) as srv:
        with pytest.raises(wlg.WlgError):
            srv.submit([request(wlg, 4, 4, 0)], couplings=[bad])
        assert srv.stats()["submitted"] == 0


def test_server_given_drawn_couplings_equal_drawn_requests(cuda):
    """Requests with their own drawn couplings given, mixed in one stream
    with requests that draw theirs: the same decoded bits either way."""
    import qec_pf_wang_landau_gb300 as wlg
    sizes = [(4, 4, 0), (5, 5, 1), (6, 6, 0), (6, 5, 1)]
    reqs = [request(wlg, X, Y, k, boundary=b, prob=0.05, intervals=4) for k, (X, Y, b) in enumerate(sizes)]
    J = [drawn_i(q.X, q.Y, q.seed, q.prob, q.sample) for q in reqs]
    with wlg.Server(0) as srv:
        ids_a = srv.submit(reqs)
        ids_b = srv.submit(reqs, couplings=J)
        ids_c = [srv.submit([q], couplings=[j] if k % 2 else None)[0] for k, (q, j) in enumerate(zip(reqs, J))]
        got = srv.wait(ids_a + ids_b + ids_c, 300)
    for a, b, c in zip(ids_a, ids_b, ids_c):
        assert same(as_tuple(got[a]), as_tuple(got[b])) and same(as_tuple(got[a]), as_tuple(got[c]))
    assert sum(got[a].status == 0 for a in ids_a) >= 2


@pytest.mark.parametrize("boundary", [0, 1])
def test_syndrome_decoding_against_exact_class_probabilities(cuda, boundary):
    """Syndrome of a drawn error -> pattern -> served request: the decoded
    class probabilities of the pattern's four classes match the exact ones
    (transfer matrix, 6x6) to Wang-Landau accuracy."""
    import qec_pf_wang_landau_gb300 as wlg
    X = Y = 6
    p = 0.08
    bn = 0.5 * np.log((1 - p) / p)
    reqs, pats, exact = [], [], []
    for k in range(3):
        S = wlg.frustration(X, Y, boundary, drawn_i(X, Y, 4242, p, k))
        J = wlg.couplings_from_syndrome(X, Y, boundary, S)
        assert np.array_equal(wlg.frustration(X, Y, boundary, J), S)
        reqs.append(request(wlg, X, Y, k, boundary=boundary, prob=p, seed=4242, intervals=6, beta=1e-4,
                            iterations=1000, pre_walkers=128, pre_intervals=32, pre_iterations=4000))
        pats.append(J)
        lz = []
        for c in "ivhc":
            Jc = J.copy()
            if c in "hc":
                Jc[X * Y:X * Y + Y] *= -1
            if c in "vc":
                Jc[0:X * Y:Y] *= -1
            cnt = O.exact_counts(Jc, X, Y, boundary)
            E = np.nonzero(cnt)[0] - 2 * X * Y
            lz.append(np.logaddexp.reduce(np.log(cnt[E + 2 * X * Y]) - bn * E))
        exact.append(np.array(lz) - np.logaddexp.reduce(lz))
    with wlg.Server(0) as srv:
        ids = srv.submit(reqs, couplings=pats)
        got = srv.wait(ids, 300)
    for i, ex in zip(ids, exact):
        d = got[i]
        assert d.status == 0
        assert np.abs(np.exp(np.array(d.log_probs)) - np.exp(ex)).max() < 0.05
