"""The serving loop (wlg_server_*): continuous batching of decoding requests.

A request is one disorder sample; the server runs its four error classes and
retires it with the classes' log-probabilities at the Nishimori temperature.
Its problems advance in short resumable main-run launches shared with every
other resident problem, so the tests check that serving changes nothing: a
served request equals the batch engine's result for the same four problems,
a request gives the same bits alone and in a mix of others arriving while it
runs, and neither the epoch length nor the memory budget matters.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CLASSES = "ivhc"


def request(wlg, X, Y, k, prob=0.06, boundary=0, **kw):
    args = dict(boundary=boundary, prob=prob, seed=777, sample=k, pre_walkers=64, pre_intervals=16,
                pre_iterations=1000, intervals=6, walkers_per_interval=4, beta=0.01, iterations=600,
                exchange_every=2)
    args.update(kw)
    return wlg.problem(X, Y, **args)


def mixed_requests(wlg, n):
    sizes = [(4, 4, 0), (5, 5, 1), (6, 6, 0), (7, 6, 1), (8, 8, 0), (10, 10, 0)]
    out = []
    for k in range(n):
        X, Y, b = sizes[k % len(sizes)]
        out.append(request(wlg, X, Y, k, boundary=b, prob=0.03 + 0.01 * (k % 7), intervals=4 if X * Y <= 25 else 6))
    return out


MISSED = (3, 5)  # WLG_ERR_NEW_ENERGY, WLG_ERR_NO_LATTICE: the pre-run missed part of the spectrum


def batch_reference(wlg, ctx, req, max_readmit=4, rounds=False):
    """The four class problems through the batch engine + class probabilities,
    with the server's re-admission: a class whose pre-run missed part of the
    spectrum is solved again with twice the pre-run iterations, up to
    max_readmit times.  rounds=True also returns the number of rounds (the
    most re-admissions of one class) and of class re-admissions."""
    out = [None] * len(CLASSES)
    todo, budget, n_rounds, n_class = list(range(len(CLASSES))), req.pre_iterations, 0, 0
    while todo:
        probs = []
        for ci in todo:
            q = wlg.Problem.from_buffer_copy(req)
            q.error_class = CLASSES[ci].encode()
            q.pre_iterations = budget
            probs.append(q)
        res = ctx.solve(probs)
        for ci, r in zip(todo, res):
            out[ci] = r
        todo = [ci for ci, r in zip(todo, res) if r[0].status in MISSED]
        if not todo or n_rounds == max_readmit:
            break
        n_rounds += 1
        n_class += len(todo)
        budget = min(2 * budget, 1 << 30)
    statuses = [r.status for r, _, _ in out]
    lz = lp = None
    if all(s == 0 for s in statuses):
        lz, lp = (np.asarray(a) for a in wlg.class_log_probs([(E, G) for _, E, G in out], req.prob))
    ret = (statuses, [r.outer_iterations for r, _, _ in out], lz, lp)
    return ret + (n_rounds, n_class) if rounds else ret


def as_tuple(d):
    return (d.status, tuple(d.outer_iterations), tuple(d.log_z), tuple(d.log_probs))


def same(a, b):
    """Bit-identical decoded results (NaN log values of failed requests match)."""
    return a[:2] == b[:2] and np.array_equal(np.array(a[2:]), np.array(b[2:]), equal_nan=True)


def test_served_requests_equal_batch_engine(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    reqs = mixed_requests(wlg, 12)
    with wlg.Server(0) as srv:
        ids = srv.submit(reqs)
        got = srv.wait(ids, 300)
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["epochs"] > 0 and st["prerun_launches"] >= 1
    ctx = wlg.Context(0)
    ok, failed = 0, []
    for i, q in zip(ids, reqs):
        d = got[i]
        statuses, outer, lz, lp = batch_reference(wlg, ctx, q)
        assert d.status == next((s for s in statuses if s != 0), 0)
        assert d.done_ms >= d.submit_ms
        if d.status != 0:
            failed.append((q.X, q.Y, d.status))
            continue
        ok += 1
        assert list(d.outer_iterations) == outer
        assert np.array_equal(np.array(d.log_z), lz)
        assert np.array_equal(np.array(d.log_probs), lp)
        assert abs(np.logaddexp.reduce(np.array(d.log_probs))) < 1e-12
    assert ok >= len(reqs) // 2, failed


def test_request_same_alone_and_in_a_mix(cuda):
    """Each request alone, then all of them arriving in a staggered stream
    while earlier ones run: identical bits, and the stream overlaps."""
    import qec_pf_wang_landau_gb300 as wlg
    reqs = mixed_requests(wlg, 10)
    alone = {}
    with wlg.Server(0) as srv:
        for k, q in enumerate(reqs):
            (i,) = srv.submit([q])
            alone[k] = as_tuple(srv.wait([i], 120)[i])
    with wlg.Server(0, epoch_outer=2) as srv:
        ids, got, peak = [], {}, 0
        for k, q in enumerate(reqs):
            ids += srv.submit([q])
            time.sleep(0.003)  # arrivals while earlier requests are resident
            peak = max(peak, srv.stats()["resident_problems"])
        t_end = time.monotonic() + 300
        while len(got) < len(ids) and time.monotonic() < t_end:
            peak = max(peak, srv.stats()["resident_problems"])
            for d in srv.poll(64, 5):
                got[int(d.id)] = d
    for k, i in enumerate(ids):
        assert same(as_tuple(got[i]), alone[k]), k
    assert peak > 4  # more than one request's problems were resident together


def test_epoch_length_and_budget_do_not_change_results(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    reqs = mixed_requests(wlg, 8)
    runs = []
    for cfg in (dict(epoch_outer=1), dict(epoch_outer=9), dict(epoch_outer=3, mem_budget_bytes=200_000,
                                                                 max_prerun_batch=2)):
        with wlg.Server(0, **cfg) as srv:
            ids = srv.submit(reqs)
            got = srv.wait(ids, 300)
            st = srv.stats()
        assert st["bytes_in_use"] <= st["bytes_budget"]
        runs.append([as_tuple(got[i]) for i in ids])
    assert all(same(a, b) and same(a, c) for a, b, c in zip(*runs))


def test_request_above_budget_is_refused(cuda):
    import qec_pf_wang_landau_gb300 as wlg
    with wlg.Server(0, mem_budget_bytes=1 << 16) as srv:
        (i,) = srv.submit([request(wlg, 16, 16, 0, intervals=8, walkers_per_interval=8)])
        d = srv.wait([i], 60)[i]
    assert d.status == 6  # WLG_ERR_OOM


def test_global_pool_form_resumes_exactly(cuda):
    """A request whose team state exceeds shared memory (one window of 256
    walkers on 10x10) keeps its FP64 log g in its arena block across epochs:
    every class stops at the same iteration with the same status (and, when
    all converge, the same log-probabilities) as the batch engine, after at
    least one suspension."""
    import qec_pf_wang_landau_gb300 as wlg
    q = request(wlg, 10, 10, 3, prob=0.05, intervals=1, walkers_per_interval=256, beta=0.05, iterations=400,
                pre_walkers=128, pre_intervals=32, pre_iterations=4000)
    ctx = wlg.Context(0)
    statuses, outer, lz, lp = batch_reference(wlg, ctx, q)
    assert ctx.stats()["main_forms"] & (1 << 3)
    with wlg.Server(0, epoch_outer=3) as srv:
        (i,) = srv.submit([q])
        d = srv.wait([i], 300)[i]
    assert d.status == next((s for s in statuses if s != 0), 0)
    assert list(d.outer_iterations) == outer
    assert max(outer) > 3
    if d.status == 0:
        assert np.array_equal(np.array(d.log_probs), lp)


def test_failure_retires_every_request_and_server_stays_usable(cuda):
    """A failure in the serving loop (injected on the host after 3 epochs; no
    GPU fault) retires every admitted and pending request with WLG_ERR_CUDA,
    later submissions fail the same way, and poll/stats/destroy keep working."""
    import qec_pf_wang_landau_gb300 as wlg
    # beta 1e-6 needs about 20 halvings of ln f, each at least one outer iteration
    reqs = [request(wlg, X, Y, k, boundary=b, beta=1e-6, intervals=4)
            for k, (X, Y, b) in enumerate([(4, 4, 0), (5, 5, 1), (6, 6, 0), (4, 4, 1), (5, 5, 0), (6, 6, 1)])]
    with wlg.Server(0, epoch_outer=1, fail_after_epochs=3) as srv:
        ids = srv.submit(reqs)
        got = srv.wait(ids, 120)
        assert all(got[i].status == 2 for i in ids)
        assert "injected failure" in wlg.lib().wlg_server_last_error(srv._h).decode()
        (late,) = srv.submit([reqs[0]])
        assert srv.wait([late], 60)[late].status == 2
        st = srv.stats()
        assert st["completed"] == len(ids) + 1 and st["epochs"] >= 3


def test_served_stitching_modes_equal_batch_engine(cuda):
    """The server's stitching mode is the context's: defined-mode decoding
    equals the batch engine with WLG_STITCH_DEFINED, bit for bit."""
    import qec_pf_wang_landau_gb300 as wlg
    reqs = mixed_requests(wlg, 4)
    ctx = wlg.Context(0)
    ctx.set_stitching(wlg.STITCH_DEFINED)
    with wlg.Server(0, stitching=wlg.STITCH_DEFINED) as srv:
        ids = srv.submit(reqs)
        got = srv.wait(ids, 300)
    for i, q in zip(ids, reqs):
        statuses, outer, lz, lp = batch_reference(wlg, ctx, q)
        d = got[i]
        assert d.status == next((s for s in statuses if s != 0), 0)
        if d.status == 0:
            assert list(d.outer_iterations) == outer
            assert np.array_equal(np.array(d.log_probs), lp)
    with pytest.raises(wlg.WlgError):
        wlg.Server(0, stitching=7)


def test_concurrent_submitters_get_the_sequential_results(cuda):
    """Four host threads submit and poll at once (ctypes releases the GIL in
    the calls): every request retires once, with the bits it gets alone."""
    import threading
    import qec_pf_wang_landau_gb300 as wlg
    reqs = [request(wlg, 4 + (k % 3), 4 + (k % 2), k, boundary=k % 2, intervals=4) for k in range(12)]
    with wlg.Server(0) as srv:
        ids = srv.submit(reqs)
        alone = srv.wait(ids, 300)
    got, errors = {}, []
    with wlg.Server(0) as srv:
        def worker(part):
            try:
                mine = srv.submit([reqs[k] for k in part])
                got.update({k: rid for k, rid in zip(part, mine)})
            except Exception as e:  # noqa: BLE001 - reported below
                errors.append(e)
        threads = [threading.Thread(target=worker, args=(list(range(w, 12, 4)),)) for w in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        done = srv.wait(list(got.values()), 300)
        assert srv.stats()["completed"] == 12
    for k, rid in got.items():
        assert same(as_tuple(done[rid]), as_tuple(alone[ids[k]])), k


def test_missed_spectrum_is_readmitted_with_a_longer_pre_run(cuda):
    """A 6x6 request whose short pre-run (16 walkers x 200 iterations) misses
    energies in classes i, v and h: each of those classes is re-admitted on
    its own as soon as it fails, with 400, 800, 1600 iterations until its
    spectrum is complete, while class c keeps running; every class's result
    equals the batch engine's at its final pre-run length, bit for bit.  With
    re-admission off the request retires with WLG_ERR_NEW_ENERGY, as the
    reference's run would abort."""
    import qec_pf_wang_landau_gb300 as wlg
    q = wlg.problem(6, 6, prob=0.1, seed=5, sample=0, pre_walkers=16, pre_intervals=16, pre_iterations=200,
                    intervals=6, walkers_per_interval=2, beta=0.05, iterations=300, exchange_every=10)
    ctx = wlg.Context(0)
    statuses, outer, lz, lp, rounds, class_readmits = batch_reference(wlg, ctx, q, rounds=True)
    assert statuses == [0, 0, 0, 0] and rounds >= 2
    first = batch_reference(wlg, ctx, q, max_readmit=0)[0]
    assert sum(s in MISSED for s in first) >= 2 and 0 in first
    with wlg.Server(0, epoch_outer=2) as srv:
        ids = srv.submit([q, q])
        got = srv.wait(ids, 300)
        st = srv.stats()
    for i in ids:
        d = got[i]
        assert d.status == 0 and d.readmissions == rounds
        assert list(d.outer_iterations) == outer
        assert np.array_equal(np.array(d.log_z), lz) and np.array_equal(np.array(d.log_probs), lp)
    assert st["readmitted"] == 2 * class_readmits and st["completed"] == 2
    with wlg.Server(0, max_readmit=-1) as srv:
        (i,) = srv.submit([q])
        d = srv.wait([i], 300)[i]
    assert d.status == next(s for s in first if s != 0) and d.readmissions == 0
