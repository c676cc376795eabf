"""Benchmark: converged disorder samples per second (and WL flips per second)
of the batched GB300 engine on the reference's matched workload.

Workload (one "step"): 6x6 periodic random-bond Ising lattices, bond flip
probability 0.04, 100 disorder samples x error classes i/v/h/c = 400
problems, seed 12345; pre-run 128 walkers, 32 coarse bins, 1000 iterations;
main run 10 windows x 3 walkers, overlap 0.25, flatness 0.8, final ln f
1e-3, 1000 WL steps per check, replica exchange every 20 checks.  Every
problem runs pre-run + main run to convergence.

value  = converged problems / (pre-run kernel + host hand-off + main-run
         kernel time), the kernels timed with CUDA events;
e2e    = the same through wlg_solve() with host buffers: problem
         descriptors in, stitched log g out, everything in the timed region;
arms   = the same 400 problems through the plain form, this engine without
         exchange (the reference's behaviour at -c 20) and the reference's own
         CUDA kernels (oracle/ref_harness.cu), untimed by the contract;
legs   = the heterogeneous batched, large-lattice, saturated large-lattice
         (152 samples, time per outer iteration against the plain form and
         the reference's kernels), converged large-lattice and serving
         workloads (summaries; full details on the line printed just before
         the headline, prefixed "detail ").
--impl reference times the CPU restatement of the reference's path (the
reference has no CPU implementation and its CUDA build needs Boost/HDF5) on
all host cores, the same 400 problems per step.
--leg NAME runs one leg alone (c3_arms: the heterogeneous workload against the
plain form and the reference's kernels, ~20 minutes).

Multi-GPU (torchrun): the problems shard by disorder sample, one shard of
400 problems per rank (weak scaling), no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(X=6, Y=6, boundary=0, prob=0.04, seed=12345, samples=100, classes="ivhc", pre_walkers=128,
                pre_intervals=32, pre_iterations=1000, intervals=10, walkers_per_interval=3, overlap=0.25, alpha=0.8,
                beta=1e-3, iterations=1000, exchange_every=20)
BYTES_PER_FLIP = 34  # log g read old + read new + write (24 B), histogram RMW (8 B), packed neighbourhood (~2 B)
# DRAM bytes (read + write) of one main-run launch of this workload, from an ncu capture of the
# bench's own launch (dram__bytes_read.sum + dram__bytes_write.sum); walker state never leaves the SM
MAIN_TRAFFIC_BYTES = 797440
METRIC = "disorder samples converged/s (6x6 pbc p=0.04, 100 samples x 4 classes)"
CPU_SAMPLE_PROBLEMS = 400  # the whole workload (samples 0-99 x ivhc)
WORKLOAD_TAG = "6x6 pbc p.04 100x4cls pre128/32/1000 I10 W3 o.25 a.8 lnf1e-3 n1000 c20"


def r4(x):
    """Floats to four significant digits, recursively (keeps the line short)."""
    if isinstance(x, float):
        return float(f"{x:.4g}") if np.isfinite(x) else None
    if isinstance(x, dict):
        return {k: r4(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [r4(v) for v in x]
    return x


def problems(rank: int = 0, exchange_mode: int = 1):
    import qec_pf_wang_landau_gb300 as wlg
    w = WORKLOAD
    out = []
    for k in range(w["samples"]):
        for c in w["classes"]:
            out.append(wlg.problem(w["X"], w["Y"], boundary=w["boundary"], prob=w["prob"], error_class=c,
                                   seed=w["seed"], sample=rank * w["samples"] + k, pre_walkers=w["pre_walkers"],
                                   pre_intervals=w["pre_intervals"], pre_iterations=w["pre_iterations"],
                                   intervals=w["intervals"], walkers_per_interval=w["walkers_per_interval"],
                                   overlap=w["overlap"], alpha=w["alpha"], beta=w["beta"],
                                   iterations=w["iterations"], exchange_every=w["exchange_every"],
                                   exchange_mode=exchange_mode))
    return out


def cpu_problems(n: int):
    import oracle as O
    w = WORKLOAD
    out = []
    for q in range(n):
        k, c = divmod(q, len(w["classes"]))
        out.append(O.OrcProblem(w["X"], w["Y"], w["boundary"], w["prob"], ord(w["classes"][c]), w["seed"], k,
                                w["pre_walkers"], w["pre_intervals"], w["pre_iterations"], w["intervals"],
                                w["walkers_per_interval"], w["overlap"], w["alpha"], w["beta"], w["iterations"],
                                w["exchange_every"], 1, 0))
    return out


def cpu_run(n: int, threads: int):
    """The oracle's C++ restatement on `threads` host threads: (problems/s, flips/s, seconds)."""
    import oracle as O
    probs = cpu_problems(n)
    t0 = time.perf_counter()
    st, outer, fl = O.run_problems(probs, threads)
    dt = time.perf_counter() - t0
    ok = int((st == 0).sum())
    return ok / dt, float(fl.sum()) / dt, dt


def plain_run():
    """The plain form (reference structure on this engine's operators) on the
    same 400 problems: (converged problems/s, seconds, kernel launches)."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = problems(0)
    t0 = time.perf_counter()
    out, launches = wlg.solve_plain(probs)
    dt = time.perf_counter() - t0
    return sum(1 for r, _, _ in out if r.status == 0) / dt, dt, launches


def reference_cuda_run():
    """The reference's own CUDA kernels (unmodified wl.cu, cubin) in its
    prerun/mainrun order, one run of 100 samples per error class.  Its
    exchange counter never advances, so at -c 20 it runs without exchange.
    Returns (converged samples/s, seconds, {class: run dict}) or None without
    the cubin."""
    import oracle as O
    if O.reference_harness() is None:
        return None
    w = WORKLOAD
    tot_ms, conv, runs = 0.0, 0, {}
    for c in w["classes"]:
        out = O.reference_run(w["X"], w["Y"], w["boundary"], w["prob"], c, w["seed"], w["samples"], w["pre_walkers"],
                              w["pre_intervals"], w["pre_iterations"], w["intervals"], w["walkers_per_interval"],
                              w["overlap"], w["alpha"], w["beta"], w["iterations"], w["exchange_every"])
        tot_ms += out["pre_ms"] + out["main_ms"]
        conv += w["samples"] if out["status"] == 0 else 0
        runs[c] = out
    return conv / (tot_ms / 1e3), tot_ms / 1e3, runs


def engine_x0_run(ctx, steps: int):
    """This engine on the same 400 problems with the reference's exchange
    behaviour at -c 20 (its counter never advances: no exchange), timed like
    the headline (pre-run + hand-off + main-run device time): the arm that
    runs the same algorithm as the reference's kernels.  Returns
    (converged samples/s, outputs of the last solve)."""
    probs = problems(0, exchange_mode=0)
    ctx.solve(probs)
    t, conv, out = 0.0, 0, None
    for _ in range(steps):
        out = ctx.solve(probs)
        st = ctx.stats()
        t += (st["pre_ms"] + st["handoff_ms"] + st["main_ms"]) / 1e3
        conv += sum(1 for r, _, _ in out if r.status == 0)
    return conv / t, out


ACCURACY_SAMPLES = 8


def _reference_curve(run, k, X, Y, I):
    """Stitched, normalised walker-0 log g of sample k from a run of the
    reference's kernels, or None."""
    import ctypes as C
    import oracle as O
    if run is None or run["status"] != 0:
        return None
    N = X * Y
    flat = np.concatenate(run["windows"][k * I:(k + 1) * I])
    Er = np.zeros(4 * N + 1, np.int32)
    Gr = np.zeros(4 * N + 1)
    n = C.c_int(0)
    rc = O.lib().orc_stitch(O.ptr(np.ascontiguousarray(flat)), O.ptr(np.ascontiguousarray(run["start"][k * I:])),
                            O.ptr(np.ascontiguousarray(run["end"][k * I:])), I, 1, X, Y, O.ptr(Er), O.ptr(Gr), len(Er),
                            C.byref(n), 0)
    return (Er[:n.value], Gr[:n.value]) if rc == 0 else None


def accuracy(arms, ref_runs):
    """log g error after normalisation against the exact density of states
    (transfer matrix over all 2^36 states) for samples 0-7 of every class:
    mean RMS and max |log g - log g_exact| over those curves, for every
    engine arm (from its timed run's own output) and for the reference's
    kernels.  And the logical-class decision of every sample (argmax over
    classes of log Z_c = logsumexp(log g_c(E) - beta_N E) at the Nishimori
    temperature) compared with the exact counts' decision.
    arms: {name: wlg_solve outputs of the 400 problems}."""
    import oracle as O
    w = WORKLOAD
    X, Y, N, I = w["X"], w["Y"], w["X"] * w["Y"], w["intervals"]
    classes = w["classes"]
    bn = 0.5 * np.log((1.0 - w["prob"]) / w["prob"])
    names = list(arms) + ["reference_cuda"]
    errs = {k: [] for k in names}
    same_sets = True
    Js = {c: O.init_interactions(X, Y, w["samples"], w["seed"], w["prob"], c) for c in classes}
    decisions = {k: [] for k in names + ["exact"]}
    for k in range(w["samples"]):
        lz = {key: [] for key in decisions}
        for ci, c in enumerate(classes):
            cnt = O.exact_counts(Js[c][k * 2 * N:(k + 1) * 2 * N], X, Y, w["boundary"])
            Ee = np.nonzero(cnt)[0] - 2 * N
            lz["exact"].append(np.logaddexp.reduce(np.log(cnt[Ee + 2 * N]) - bn * Ee))
            curves = {}
            for name, out in arms.items():
                r, E, G = out[k * len(classes) + ci]
                curves[name] = (E, G) if r.status == 0 else None
            curves["reference_cuda"] = _reference_curve(None if ref_runs is None else ref_runs.get(c), k, X, Y, I)
            for name, cv in curves.items():
                lz[name].append(np.logaddexp.reduce(cv[1] - bn * cv[0]) if cv is not None else np.nan)
                if k < ACCURACY_SAMPLES and cv is not None:
                    if name != "reference_cuda":
                        same_sets &= set(cv[0].tolist()) == set(Ee.tolist())
                    err = cv[1] - np.log(cnt[cv[0] + 2 * N])
                    errs[name].append((float(np.sqrt(np.mean(err ** 2))), float(np.abs(err).max())))
        for key, v in lz.items():
            decisions[key].append(int(np.argmax(v)) if np.all(np.isfinite(v)) else -1)
    d = {key: np.array(v) for key, v in decisions.items()}
    return {"exact": "transfer matrix, 2^36 states", "curves": f"samples 0-{ACCURACY_SAMPLES - 1} x {classes}",
            "rms": {k: float(np.mean([a for a, _ in v])) for k, v in errs.items() if v},
            "max": {k: float(max(b for _, b in v)) for k, v in errs.items() if v},
            "engine_sets_exact": bool(same_sets),
            "class_decisions_equal_exact": {k: int(np.sum((d[k] == d["exact"]) & (d[k] >= 0))) for k in names},
            "samples": w["samples"],
            "exact_class_counts": {c: int(np.sum(d["exact"] == ci)) for ci, c in enumerate(classes)}}


SERVING = dict(rate=200.0, seconds=1.0, side_min=4, side_max=16, prob_min=0.02, prob_max=0.12, beta=1e-6,
               walkers_per_interval=4, wait_s=180.0, seed=2026)


def serving_requests(n_max: int = 100000):
    """Poisson arrival times and decoding requests of the serving workload:
    square periodic lattices with side uniform in {4..16}, p uniform in
    [0.02, 0.12], ln f 1e-6, windows scaled with N (N/16, 4..16), 4 walkers
    each, pre-run 128 walkers x 400 N iterations; all four classes per
    request (the server runs them)."""
    import qec_pf_wang_landau_gb300 as wlg
    c = SERVING
    rng = np.random.default_rng(c["seed"])
    t, arrivals, reqs = 0.0, [], []
    while len(reqs) < n_max:
        t += rng.exponential(1.0 / c["rate"])
        if t > c["seconds"]:
            break
        L = int(rng.integers(c["side_min"], c["side_max"] + 1))
        N = L * L
        arrivals.append(t)
        reqs.append(wlg.problem(L, L, prob=float(rng.uniform(c["prob_min"], c["prob_max"])), seed=c["seed"],
                                sample=len(reqs), pre_walkers=128, pre_intervals=32, pre_iterations=400 * N,
                                intervals=int(min(16, max(4, N // 16))), walkers_per_interval=c["walkers_per_interval"],
                                overlap=0.25, alpha=0.8, beta=c["beta"], iterations=1000, exchange_every=10))
    return arrivals, reqs


def serving_run():
    """The serving workload through wlg_server: requests submitted at their
    Poisson arrival times, latency = retirement - submission (server clock)."""
    import qec_pf_wang_landau_gb300 as wlg
    arrivals, reqs = serving_requests()
    got, ids = {}, []
    with wlg.Server(0) as srv:
        t0 = time.perf_counter()
        for a, q in zip(arrivals, reqs):
            delay = t0 + a - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids += srv.submit([q])
            for d in srv.poll(256, 0):
                got[int(d.id)] = d
        while len(got) < len(ids) and time.perf_counter() - t0 < SERVING["wait_s"]:
            for d in srv.poll(256, 50):
                got[int(d.id)] = d
        st = srv.stats()
    done = [got[i] for i in ids if i in got]
    lat = np.array([d.done_ms - d.submit_ms for d in done]) if done else np.zeros(1)
    side = {i: q.X for i, q in zip(ids, reqs)}
    slow = []  # the longest requests: what their latency is made of
    for d in sorted(done, key=lambda d: d.submit_ms - d.done_ms)[:3]:
        slow.append({"latency_s": (d.done_ms - d.submit_ms) / 1e3, "side": side[int(d.id)],
                     "outer_ivhc": list(d.outer_iterations), "readmissions": d.readmissions, "status": d.status})
    span_s = (max(d.done_ms for d in done) - min(d.submit_ms for d in done)) / 1e3 if done else float("nan")
    statuses = {}
    for d in done:
        statuses[str(d.status)] = statuses.get(str(d.status), 0) + 1
    return {"workload": "Poisson 200 req/s for 1 s, side U{4..16} periodic, p U[0.02,0.12], ln f 1e-6, "
                        "4 classes per request, W=4, I=N/16 in [4,16]",
            "requests": len(ids), "retired": len(done), "retired_ok": statuses.get("0", 0), "status_counts": statuses,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "throughput_req_s": len(done) / span_s if done else 0.0,
            "epochs": st["epochs"], "prerun_launches": st["prerun_launches"], "readmitted": st["readmitted"],
            "requests_readmitted": sum(1 for d in done if d.readmissions > 0), "slowest": slow,
            "note": f"requests not retired within {SERVING['wait_s']:.0f} s are left out of the percentiles"}


BATCHED = dict(samples=2000, sides=(4, 6, 8, 10, 12), prob_min=0.02, prob_max=0.12, beta=1e-6, seed=31337)


def batched_problems():
    """The heterogeneous batched workload: 2000 disorder samples, side
    uniform in {4,6,8,10,12}, boundary periodic/open 50/50, p uniform in
    [0.02, 0.12], class uniform over i/v/h/c, windows 8..32 scaled with N,
    4 walkers each, overlap 0.25, flatness 0.8, ln f 1e-6; per-sample
    parameters from a seeded host generator, disorder from Philox."""
    import qec_pf_wang_landau_gb300 as wlg
    c = BATCHED
    rng = np.random.default_rng(c["seed"])
    out = []
    for k in range(c["samples"]):
        L = int(rng.choice(c["sides"]))
        N = L * L
        out.append(wlg.problem(L, L, boundary=int(rng.integers(0, 2)), prob=float(rng.uniform(c["prob_min"], c["prob_max"])),
                               error_class="ivhc"[int(rng.integers(0, 4))], seed=c["seed"], sample=k, pre_walkers=128,
                               pre_intervals=32, pre_iterations=100 * N, intervals=int(min(32, max(8, N // 8))),
                               walkers_per_interval=4, overlap=0.25, alpha=0.8, beta=c["beta"], iterations=1000,
                               exchange_every=10))
    return out


def batched_run():
    """The heterogeneous batch in one wlg_solve call: converged samples/s."""
    import qec_pf_wang_landau_gb300 as wlg
    probs = batched_problems()
    ctx = wlg.Context(0)
    t0 = time.perf_counter()
    out = ctx.solve(probs)
    wall = time.perf_counter() - t0
    st = ctx.stats()
    dev_s = (st["pre_ms"] + st["handoff_ms"] + st["main_ms"]) / 1e3
    counts = {}
    for r, _, _ in out:
        counts[str(r.status)] = counts.get(str(r.status), 0) + 1
    flips = sum(r.flips for r, _, _ in out)
    return {"workload": "2000 samples, side U{4,6,8,10,12}, open/periodic 50/50, p U[0.02,0.12], class U{ivhc}, "
                        "I = N/8 in [8,32], W=4, o=0.25, alpha=0.8, ln f 1e-6, exchange every 10",
            "value": counts.get("0", 0) / dev_s, "unit": "samples/s", "e2e_samples_per_s": counts.get("0", 0) / wall,
            "status_counts": counts, "flips_per_s": flips / (st["main_ms"] / 1e3), "pre_ms": st["pre_ms"],
            "main_ms": st["main_ms"], "main_forms": st["main_forms"], "kernel_launches": st["kernel_launches"],
            **critical_path(ctx, probs, out), "accuracy": batched_accuracy(probs, out)}


def critical_path(ctx, probs, out):
    """Where a batch's main-run time goes, from each problem's start and end
    on the device clock: the longest single problem (its own serial chain of
    outer iterations; no schedule can finish the batch sooner), when problems
    finish, and how busy the teams were (sum of problem spans / (main-run
    time x most problems running at once))."""
    t0, t1 = ctx.main_times()
    ran = t0 >= 0
    if not np.any(ran):
        return {}
    span = np.where(ran, t1 - t0, 0.0)
    q = int(np.argmax(span))
    r = out[q][0]
    ev = sorted([(a, 1) for a in t0[ran]] + [(b, -1) for b in t1[ran]])
    live = peak = 0
    for _, d in ev:
        live += d
        peak = max(peak, live)
    by_side, start_by_side = {}, {}
    for p, sp, a, ok in zip(probs, span, t0, ran):
        if ok:
            by_side.setdefault(f"{p.X}x{p.Y}", []).append(sp)
            start_by_side.setdefault(f"{p.X}x{p.Y}", []).append(a)
    z = int(np.argmax(np.where(ran, t1, -1.0)))  # the problem that ends the main run
    return {"critical_path_ms": float(span[q]),
            "critical_problem": {"side": probs[q].X, "boundary": probs[q].boundary, "windows": probs[q].intervals,
                                 "outer_iterations": int(r.outer_iterations), "start_ms": float(t0[q]),
                                 "us_per_outer": 1e3 * float(span[q]) / max(int(r.outer_iterations), 1)},
            "last_problem": {"side": probs[z].X, "start_ms": float(t0[z]), "span_ms": float(span[z]),
                             "outer_iterations": int(out[z][0].outer_iterations)},
            "start_ms_max_by_side": {k: float(max(v)) for k, v in sorted(start_by_side.items())},
            "last_end_ms": float(t1[ran].max()),
            "end_ms_p50_p90": [float(np.percentile(t1[ran], 50)), float(np.percentile(t1[ran], 90))],
            "span_ms_max_by_side": {k: float(max(v)) for k, v in sorted(by_side.items())},
            "concurrent_peak": peak,
            "team_busy_frac": float(span.sum() / (peak * t1[ran].max()))}


# curves scored per side: a periodic 12x12 curve takes tens of seconds of
# host time (2^143 states through the transfer matrix), the others well under one
BATCHED_ACCURACY_PER_SIDE = {4: 4, 6: 4, 8: 4, 10: 4, 12: 2}


def batched_accuracy(probs, out):
    """log g error of the batched leg's own output against the exact density
    of states (transfer matrix, up to 2^144 states) for the first converged
    samples of every side: RMS and max |log g - log g_exact| after
    normalisation, per side."""
    import oracle as O
    res = {}
    for L, cap in BATCHED_ACCURACY_PER_SIDE.items():
        errs, same = [], True
        for p, (r, E, G) in zip(probs, out):
            if p.X != L or r.status != 0 or len(errs) == cap:
                continue
            N = L * L
            J = O.init_interactions(L, L, p.sample + 1, p.seed, p.prob, p.error_class.decode())[p.sample * 2 * N:]
            cnt = O.exact_counts(J, L, L, p.boundary)
            same &= set(E.tolist()) == set((np.nonzero(cnt)[0] - 2 * N).tolist())
            err = G - np.log(cnt[E + 2 * N])
            errs.append((float(np.sqrt(np.mean(err ** 2))), float(np.abs(err).max())))
        if errs:
            res[f"{L}x{L}"] = {"curves": len(errs), "rms_mean": float(np.mean([a for a, _ in errs])),
                               "max_abs": float(max(b for _, b in errs)), "energy_sets_exact": bool(same)}
    return res


C3_ARMS = dict(seed=7000, sides=(4, 6, 8, 10, 12), per_group=3, beta=1e-6)


def c3_group_problems(exchange_mode: int, per_group: int, sides=None):
    """A subset of the heterogeneous workload laid out as the reference's
    programs would run it: one group per (side, boundary, class), each group a
    run of samples 0..R-1 with its own bond probability (uniform in
    [0.02, 0.12]) and seed; windows N/8 in [8, 32], 4 walkers, overlap 0.25,
    flatness 0.8, ln f 1e-6, exchange every 10 iterations."""
    import qec_pf_wang_landau_gb300 as wlg
    c = C3_ARMS
    rng = np.random.default_rng(c["seed"])
    out, g = [], 0
    for L in (sides or c["sides"]):
        for b in (0, 1):
            for cls in "ivhc":
                prob = float(np.float32(rng.uniform(0.02, 0.12)))
                N = L * L
                for k in range(per_group):
                    out.append(wlg.problem(L, L, boundary=b, prob=prob, error_class=cls, seed=c["seed"] + 100 * g,
                                           sample=k, pre_walkers=128, pre_intervals=32, pre_iterations=100 * N,
                                           intervals=int(min(32, max(8, N // 8))), walkers_per_interval=4,
                                           overlap=0.25, alpha=0.8, beta=c["beta"], iterations=1000,
                                           exchange_every=10, exchange_mode=exchange_mode))
                g += 1
    return out


def _groups(probs):
    """Runs of the reference's programs: consecutive problems that share all but the sample."""
    runs = []
    for q, p in enumerate(probs):
        if p.sample == 0:
            runs.append([q])
        else:
            runs[-1].append(q)
    return runs


def _exact_rms(p, E, G):
    import oracle as O
    N = p.X * p.Y
    J = O.init_interactions(p.X, p.Y, p.sample + 1, p.seed, p.prob, p.error_class.decode())[p.sample * 2 * N:]
    cnt = O.exact_counts(J, p.X, p.Y, p.boundary)
    err = G - np.log(cnt[E + 2 * N])
    return float(np.sqrt(np.mean(err ** 2))), set(E.tolist()) == set((np.nonzero(cnt)[0] - 2 * N).tolist())


def c3_arms_run(per_group=None, sides=None, ref_budget_s=600.0):
    """The heterogeneous workload's comparison (grouped subset, c3_group_problems):
    this engine batched (every group in one wlg_solve; exchange every 10, and
    with the reference's exchange behaviour, mode 0), the plain form (the
    reference's structure on this engine's operators, one run per group) and
    the reference's own kernels (one prerun + mainrun per group, as its
    programs run; no exchange, its counter never advances).  Converged
    samples/s of each, and the log g RMS against exact counts of each arm on
    the same curves (sample 0 of every group up to 10x10, open 12x12)."""
    import qec_pf_wang_landau_gb300 as wlg
    import oracle as O
    R = per_group or C3_ARMS["per_group"]
    probs = {m: c3_group_problems(m, R, sides) for m in (0, 1)}
    ctx = wlg.Context(0)
    res, outs = {}, {}
    for m, name in ((1, "engine"), (0, "engine_x0")):
        ctx.solve(probs[m][:8])  # warm the context's buffers
        t0 = time.perf_counter()
        out = ctx.solve(probs[m])
        wall = time.perf_counter() - t0
        st = ctx.stats()
        ok = sum(1 for r, _, _ in out if r.status == 0)
        res[name] = {"value": ok / ((st["pre_ms"] + st["handoff_ms"] + st["main_ms"]) / 1e3), "wall_s": wall,
                     "e2e": ok / wall, "converged": ok, **{k: v for k, v in critical_path(ctx, probs[m], out).items()
                                                           if k in ("critical_path_ms", "last_end_ms")}}
        outs[name] = out
    t0 = time.perf_counter()
    out_p, launches = wlg.solve_plain(probs[0])
    wall = time.perf_counter() - t0
    ok = sum(1 for r, _, _ in out_p if r.status == 0)
    res["plain"] = {"value": ok / wall, "wall_s": wall, "converged": ok, "kernel_launches": launches}
    outs["plain"] = out_p
    if O.reference_harness() is not None:
        ref_out = [None] * len(probs[0])
        tot_ms, ok, done_groups = 0.0, 0, 0
        runs = _groups(probs[0])
        for run in runs:
            if tot_ms / 1e3 > ref_budget_s:
                break
            p = probs[0][run[0]]
            o = O.reference_run(p.X, p.Y, p.boundary, p.prob, p.error_class.decode(), p.seed, len(run),
                                p.pre_walkers, p.pre_intervals, p.pre_iterations, p.intervals,
                                p.walkers_per_interval, p.overlap, p.alpha, p.beta, p.iterations, p.exchange_every)
            tot_ms += o["pre_ms"] + o["main_ms"]
            done_groups += 1
            if o["status"] == 0:
                ok += len(run)
                for k, q in enumerate(run):
                    ref_out[q] = _reference_curve(o, k, p.X, p.Y, p.intervals)
        res["reference_cuda"] = {"value": ok / (tot_ms / 1e3), "seconds": tot_ms / 1e3, "converged": ok,
                                 "groups_run": done_groups, "groups": len(runs)}
        outs["reference_cuda"] = ref_out
    # accuracy on the same curves
    acc = {k: [] for k in outs}
    for run in _groups(probs[0]):
        q = run[0]
        p = probs[0][q]
        if p.X > 12 or (p.X == 12 and p.boundary == 0):
            continue
        curves = {}
        for k, o in outs.items():
            if k == "reference_cuda":
                curves[k] = o[q]
            else:
                r, E, G = o[q]
                curves[k] = (E, G) if r.status == 0 else None
        if any(v is None for v in curves.values()):
            continue
        for k, (E, G) in curves.items():
            acc[k].append(_exact_rms(p, E, G)[0])
    for k, v in acc.items():
        res[k]["rms"] = float(np.mean(v)) if v else None
        res[k]["curves"] = len(v)
    res["workload"] = (f"{len(_groups(probs[0]))} groups (side x boundary x class) x {R} samples, p U[0.02,0.12] per "
                       f"group, I=N/8 in [8,32], W=4, o=0.25, a=0.8, ln f 1e-6, exchange every 10")
    if "reference_cuda" in res:
        res["engine_x0_over_reference_cuda"] = res["engine_x0"]["value"] / res["reference_cuda"]["value"]
    res["engine_over_plain"] = res["engine"]["value"] / res["plain"]["value"]
    return res


# one class by default: the reference's kernels take about 50 s per class at
# ln f 1e-5 and several minutes at 1e-4 or below over four classes
LARGE_CONV = dict(side=16, samples=1, classes="v", prob=0.10, seed=4343, beta=1e-5)


def large_converged_run(side=None, samples=None, beta=None, classes=None):
    """The large-lattice workload run to convergence on a bounded sample:
    side x side periodic, p = 0.10, all four classes, 64 windows x 8 walkers,
    overlap 0.3, exchange every 10.  This engine (exchange every 10, and
    mode 0), the plain form and the reference's own kernels (one run per
    class, no exchange) on the same problems; there is no exact density of
    states at this size, so each arm's normalised log g is compared with the
    reference kernels' on their common energies (RMS difference)."""
    import qec_pf_wang_landau_gb300 as wlg
    import oracle as O
    c = dict(LARGE_CONV)
    c.update({k: v for k, v in (("side", side), ("samples", samples), ("beta", beta), ("classes", classes))
              if v is not None})
    L, N = c["side"], c["side"] ** 2

    def mk(m):
        return [wlg.problem(L, L, prob=c["prob"], error_class=cl, seed=c["seed"], sample=k, pre_walkers=128,
                            pre_intervals=128, pre_iterations=1000 * N, intervals=64, walkers_per_interval=8,
                            overlap=0.3, alpha=0.8, beta=c["beta"], iterations=1000, exchange_every=10,
                            exchange_mode=m) for cl in c["classes"] for k in range(c["samples"])]
    probs = {m: mk(m) for m in (0, 1)}
    ctx = wlg.Context(0)
    res, curves = {}, {}
    for m, name in ((1, "engine"), (0, "engine_x0")):
        out = ctx.solve(probs[m])
        st = ctx.stats()
        ok = sum(1 for r, _, _ in out if r.status == 0)
        res[name] = {"value": ok / ((st["pre_ms"] + st["handoff_ms"] + st["main_ms"]) / 1e3), "converged": ok,
                     "main_ms": st["main_ms"], "outer_max": max(r.outer_iterations for r, _, _ in out)}
        curves[name] = [(E, G) if r.status == 0 else None for r, E, G in out]
    t0 = time.perf_counter()
    out_p, _ = wlg.solve_plain(probs[0])
    wall = time.perf_counter() - t0
    ok = sum(1 for r, _, _ in out_p if r.status == 0)
    res["plain"] = {"value": ok / wall, "seconds": wall, "converged": ok}
    curves["plain"] = [(E, G) if r.status == 0 else None for r, E, G in out_p]
    if O.reference_harness() is not None:
        tot, ok, ref = 0.0, 0, []
        for cl in c["classes"]:
            o = O.reference_run(L, L, 0, c["prob"], cl, c["seed"], c["samples"], 128, 128, 1000 * N, 64, 8, 0.3, 0.8,
                                c["beta"], 1000, 10)
            tot += o["pre_ms"] + o["main_ms"]
            ok += c["samples"] if o["status"] == 0 else 0
            ref += [_reference_curve(o, k, L, L, 64) for k in range(c["samples"])]
        res["reference_cuda"] = {"value": ok / (tot / 1e3), "seconds": tot / 1e3, "converged": ok}
        for name in ("engine", "engine_x0", "plain"):
            d = []
            for a, b in zip(curves[name], ref):
                if a is None or b is None:
                    continue
                common, ia, ib = np.intersect1d(a[0], b[0], return_indices=True)
                d.append(float(np.sqrt(np.mean((a[1][ia] - b[1][ib]) ** 2))))
            res[name]["rms_vs_reference"] = float(np.mean(d)) if d else None
            res[name]["curves"] = len(d)
        res["engine_x0_over_reference_cuda"] = res["engine_x0"]["value"] / res["reference_cuda"]["value"]
    res["engine_over_plain"] = res["engine"]["value"] / res["plain"]["value"]
    res["workload"] = (f"{L}x{L} periodic p={c['prob']}, {c['samples']} samples x classes {c['classes']}, I=64 W=8 "
                       f"o=0.3 a=0.8, ln f {c['beta']:g}, exchange every 10, pre-run 128 x 1000 N")
    return res


def large_saturated_run(sides=(16, 24), samples=152, caps=(10, 40)):
    """Throughput of the large-lattice workload with the GPU full: `samples`
    disorder samples (152: one 512-thread team per SM for this engine; 152 x 64
    blocks for the reference's kernels), class v, p = 0.10, 64 windows x 8
    walkers, overlap 0.3, no exchange in every arm (the reference's behaviour
    at -c 10), each run capped at caps[0] and then caps[1] outer iterations
    (ln f 1e-8 is never reached, so no sample finishes).  The difference of
    the two runs' times over the difference of the caps is the time of one
    outer iteration of all samples, pre-run and set-up cancelled: with the
    same algorithm the iterations to convergence are the same in every arm,
    so its ratio between arms is their throughput ratio."""
    import qec_pf_wang_landau_gb300 as wlg
    import oracle as O
    res = {"workload": f"{samples} samples x class v, p=0.10, I=64 W=8 o=0.3, no exchange, outer capped at {caps}"}
    for L in sides:
        N = L * L

        def probs(cap):
            return [wlg.problem(L, L, prob=0.10, error_class="v", seed=5151, sample=k, pre_walkers=128,
                                pre_intervals=128, pre_iterations=1000 * N, intervals=64, walkers_per_interval=8,
                                overlap=0.3, alpha=0.8, beta=1e-8, iterations=1000, exchange_every=10,
                                exchange_mode=0, max_outer=cap) for k in range(samples)]
        ctx = wlg.Context(0)
        eng, pl, rf = [], [], []
        for cap in caps:
            out = ctx.solve_raw(probs(cap))
            eng.append((ctx.stats()["main_ms"], max(r.outer_iterations for r, _, _, _ in out)))
            t0 = time.perf_counter()
            outp, _ = wlg.solve_plain(probs(cap))
            pl.append((1e3 * (time.perf_counter() - t0), max(r.outer_iterations for r, _, _ in outp)))
            if O.reference_harness() is not None:
                o = O.reference_run(L, L, 0, 0.10, "v", 5151, samples, 128, 128, 1000 * N, 64, 8, 0.3, 0.8, 1e-8, 1000,
                                    10, max_outer=cap, want_raw=False)
                rf.append((o["main_ms"], o["outer"]))

        def per_outer(v):
            return (v[1][0] - v[0][0]) / max(v[1][1] - v[0][1], 1)
        r = {"engine_ms_per_outer": per_outer(eng), "plain_ms_per_outer": per_outer(pl),
             "outer": [eng[0][1], eng[1][1]]}
        if rf:
            r["reference_ms_per_outer"] = per_outer(rf)
            r["reference_over_engine"] = r["reference_ms_per_outer"] / r["engine_ms_per_outer"]
            r["reference_outer"] = [rf[0][1], rf[1][1]]
        r["plain_over_engine"] = r["plain_ms_per_outer"] / r["engine_ms_per_outer"]
        res[f"{L}x{L}"] = r
        print("partial " + json.dumps(r4({f"{L}x{L}": r})), flush=True)
    return res


LARGE = dict(sides=(16, 24), samples=38, prob=0.10, seed=4242, max_outer=10)


def large_run():
    """The large-lattice workload (16x16 and 24x24 periodic, p = 0.10, all four
    classes, 64 windows x 8 walkers, overlap 0.3, exchange every 10, ln f 1e-8),
    bounded: one wave of 38 samples x 4 classes per side, each capped at 10
    outer iterations (a run to ln f 1e-8 takes hours).  Reports the WL flip
    rate and the step time of the 512-thread teams."""
    import qec_pf_wang_landau_gb300 as wlg
    c = LARGE
    out = {"workload": "16x16 and 24x24 periodic, p=0.10, classes ivhc, I=64 x W=8, o=0.3, alpha=0.8, ln f 1e-8, "
                       "exchange every 10; 38 samples x 4 classes per side, capped at 10 outer iterations"}
    ctx = wlg.Context(0)
    for L in c["sides"]:
        N = L * L
        probs = [wlg.problem(L, L, prob=c["prob"], error_class=cl, seed=c["seed"], sample=k, pre_walkers=128,
                             pre_intervals=128, pre_iterations=100 * N, intervals=64, walkers_per_interval=8,
                             overlap=0.3, alpha=0.8, beta=1e-8, iterations=1000, exchange_every=10,
                             max_outer=c["max_outer"]) for k in range(c["samples"]) for cl in "ivhc"]
        res = ctx.solve_raw(probs)
        st = ctx.stats()
        flips = sum(r.flips for r, _, _, _ in res)
        outer = max(r.outer_iterations for r, _, _, _ in res)
        out[f"{L}x{L}"] = {"problems": len(probs), "flips_per_s": flips / (st["main_ms"] / 1e3),
                           "main_ms": st["main_ms"], "pre_ms": st["pre_ms"],
                           "us_per_step": st["main_ms"] * 1e3 / (outer * 1000), "main_forms": st["main_forms"],
                           "ran": sum(1 for r, _, _, _ in res if r.status in (0, 7))}
    return out


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self, device_index: int = 0):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device_index):
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.remove(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(torch, buf):
    buf.add_(1)  # 512 MiB read+write, far beyond the 129 MB L2


def reduce_over_ranks(dist, times, counts, device):
    """Whole-job figures of a sharded run: the slowest rank's times, the
    sum of every rank's counts (samples, flips).  No data-path collective:
    ranks solve disjoint samples and meet only here."""
    import torch
    tt = torch.tensor(times, dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    cc = torch.tensor(counts, dtype=torch.float64, device=device)
    dist.all_reduce(cc, op=dist.ReduceOp.SUM)
    return tt.tolist(), [int(v) for v in cc.tolist()]


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    import torch
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, ws, dist


# The extra legs start only while the run is younger than this (seconds), so
# that a slow box still prints the headline line in bounded time.
LEG_BUDGET_S = 330.0


def run_ours(args):
    import torch
    import qec_pf_wang_landau_gb300 as wlg
    t_run = time.perf_counter()
    wlg.build()
    rank, ws, dist = dist_init()
    dev = torch.cuda.current_device()
    ctx = wlg.Context(dev)
    probs = problems(rank)
    flush = torch.zeros(128 * 1024 * 1024, dtype=torch.int32, device="cuda")
    tuning = ctx.autotune(probs, max_outer=3)  # teams per CTA, kept by the context (untimed)
    for _ in range(args.warmup):
        ctx.solve(probs)
    torch.cuda.synchronize()
    sampler = ClockSampler()
    if rank == 0:
        sampler.start()
    dev_ms, e2e_s, converged, flips, main_ms = [], [], 0, 0, []
    h2d = d2h = launches = 0
    for _ in range(args.steps):
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        out = ctx.solve(probs)  # wlg_solve synchronises its own stream before returning
        last_out = out
        e2e_s.append(time.perf_counter() - t0)
        st = ctx.stats()
        dev_ms.append(st["pre_ms"] + st["handoff_ms"] + st["main_ms"])
        main_ms.append(st["main_ms"])
        converged += sum(1 for r, _, _ in out if r.status == 0)
        flips += sum(r.flips for r, _, _ in out)
        h2d, d2h, launches = st["h2d_bytes"], st["d2h_bytes"], launches + st["kernel_launches"]
    torch.cuda.synchronize()
    clocks = sampler.stop(dev) if rank == 0 else None
    t_dev = sum(dev_ms) / 1e3
    t_e2e = sum(e2e_s)
    t_main = sum(main_ms) / 1e3
    if dist is not None:
        (t_dev, t_e2e, t_main), (converged, flips) = reduce_over_ranks(dist, [t_dev, t_e2e, t_main],
                                                                       [converged, flips], "cuda")
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return None
    # the single-GPU comparison arms and legs run at N = 1 only (the CPU
    # baseline is a rank-0, N = 1 figure; at N > 1 they would hold every GPU)
    single = ws == 1
    peaks, peak_kind = measured_peaks()
    achieved = BYTES_PER_FLIP * flips / max(t_main, 1e-12) / 1e9
    value = converged / t_dev
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "samples/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32+f64",
        "data": "synthetic, seeded Philox",
        "config": {"workload": WORKLOAD_TAG, "l2": "flushed",
                   "teams_per_cta": {f"f{t['form']}/t{t['team']}": t["per_cta"] for t in tuning}},
        "e2e": {"value": converged / t_e2e, "unit": "samples/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": MAIN_TRAFFIC_BYTES,
                     "peak_kind": peak_kind},
        "flips_per_s": flips / t_main,
    }
    if clocks is not None:
        line["clocks"] = {k: clocks[k] for k in ("sm_mhz", "sm_max_mhz", "reasons")}
    if not single:
        return r4(line)
    cpu_pps, cpu_fps, cpu_s = cpu_run(CPU_SAMPLE_PROBLEMS, os.cpu_count() or 1)
    line["cpu_baseline"] = {"value": cpu_pps, "unit": "samples/s", "cores": os.cpu_count(), "kind": "port",
                            "sample": f"{CPU_SAMPLE_PROBLEMS} problems"}
    # comparison arms on the same 400 problems (samples/s, converged; device or wall time as stated)
    plain_pps, plain_s, plain_launches = plain_run()
    ref_cuda = reference_cuda_run()
    x0_pps, x0_out = engine_x0_run(ctx, 3)
    # arms (samples/s): plain form, this engine without exchange (x0, the
    # reference's behaviour at -c 20), the reference's kernels (ref); ratios
    arms = {"plain": plain_pps, "x0": x0_pps}
    if ref_cuda is not None:
        arms["ref"] = ref_cuda[0]
        arms["x0/ref"] = x0_pps / ref_cuda[0]
    arms["v/plain"] = value / plain_pps
    line["arms"] = arms
    acc = accuracy({"engine": last_out, "engine_x0": x0_out}, ref_cuda[2] if ref_cuda is not None else None)
    short = {"engine": "eng", "engine_x0": "x0", "reference_cuda": "ref"}
    line["accuracy"] = {"rms": {short[k]: v for k, v in acc["rms"].items()},
                        "cls_ok": {short[k]: v for k, v in acc["class_decisions_equal_exact"].items()},
                        "of": acc["samples"], "sets_ok": acc["engine_sets_exact"]}
    sec = secondary_ceilings(achieved, flips / t_main)
    detail = {"plain": {"seconds": plain_s, "kernel_launches": plain_launches,
                        "what": "same 400 problems, reference structure on this engine's operator kernels"},
              "reference_cuda": None if ref_cuda is None else {
                  "seconds": ref_cuda[1], "what": "the reference's own kernels (unmodified wl.cu for sm_103a) in its "
                                                  "prerun/mainrun order; no exchange at -c 20 (its counter never "
                                                  "advances)"},
              "engine_x0": "this engine, exchange_mode 0 (the reference's behaviour at -c 20), device time",
              "accuracy": acc, **sec}
    line["roofline"]["smem_frac"] = sec["roofline_smem"]["frac"]
    if not args.no_extra:
        legs = {name: run_leg(fn, t_run) for name, fn in (("batched", batched_run), ("large", large_run),
                                                          ("large_saturated", large_saturated_run),
                                                          ("large_converged", large_converged_run),
                                                          ("serving", serving_run))}
        detail.update(legs)
        line["legs"] = legs_summary(legs)
    print("detail " + json.dumps(r4(detail)), flush=True)
    return r4(line)


def run_leg(fn, t_run=None):
    """One extra leg; a leg that fails is reported as {"error": ...} so that
    the headline line is still printed, and a leg that would start after
    LEG_BUDGET_S seconds of the run (from t_run) is skipped and reported so."""
    if t_run is not None and time.perf_counter() - t_run > LEG_BUDGET_S:
        return {"error": f"skipped: the run passed {LEG_BUDGET_S:.0f} s"}
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 - any failure of a leg is reported, not raised
        print(f"leg {fn.__name__} failed: {type(e).__name__}: {e}", file=sys.stderr, flush=True)
        return {"error": f"{type(e).__name__}: {e}"[:200]}


def legs_summary(legs):
    """A few numbers per extra leg for the headline line: samples/s, times in
    s, flip rates in G/s (gflips, per lattice side); x0 = this engine without
    exchange, ref = the reference's kernels; batched crit = critical path /
    main-run time; lconv rms = the engine's log g RMS against ref."""
    out = {}
    failed = [k for k, v in legs.items() if isinstance(v, dict) and "error" in v]
    if failed:
        out["failed"] = failed
    legs = {k: v for k, v in legs.items() if k not in failed}
    b = legs.get("batched")
    if b:
        crit, main = b.get("critical_path_ms"), b.get("main_ms")
        out["batched"] = {"v": b["value"], "ok": b["status_counts"].get("0", 0),
                          "rms": max(v["rms_mean"] for v in b["accuracy"].values()) if b["accuracy"] else None,
                          "main_s": main / 1e3 if main else None,
                          "crit": crit / main if crit and main else None}
    g = legs.get("large")
    if g:
        out["gflips"] = [v["flips_per_s"] / 1e9 for v in g.values() if isinstance(v, dict)]
    t = legs.get("large_saturated")
    if t:
        # per side, time per outer iteration with the GPU full, no exchange: [reference / engine, plain / engine]
        out["sat"] = [[v.get("reference_over_engine"), v["plain_over_engine"]] for v in t.values()
                      if isinstance(v, dict)]
    c = legs.get("large_converged")
    if c:
        out["lconv"] = {"v": c["engine"]["value"], "x0": c["engine_x0"]["value"]}
        if "reference_cuda" in c:
            out["lconv"]["ref"] = c["reference_cuda"]["value"]
            out["lconv"]["rms"] = c["engine"].get("rms_vs_reference")
    v = legs.get("serving")
    if v:
        out["serving"] = {"ok": f'{v["retired_ok"]}/{v["requests"]}', "readm": v["requests_readmitted"],
                          "p99_s": v["p99_ms"] / 1e3}
    return out


def secondary_ceilings(achieved_gbs, flips_per_s):
    """The rates the WL step depends on besides HBM, measured on this device
    after the timed region (wlg_measure_peaks): the main run's 34 B per flip
    against shared-memory bandwidth (the level that holds its walker state),
    and the step rates that Philox draws (two per step) and FP64 exp + log
    (one each per step in the reference's formulation) would allow alone."""
    import qec_pf_wang_landau_gb300 as wlg
    pk = wlg.measure_peaks(0)
    fp64_step = 1.0 / (1.0 / pk["exp_f64_per_s"] + 1.0 / pk["log_f64_per_s"])
    return {
        "roofline_smem": {"achieved": achieved_gbs, "peak": pk["smem_gbs"], "unit": "GB/s",
                          "frac": achieved_gbs / pk["smem_gbs"], "peak_kind": "measured (wlg_measure_peaks)"},
        "secondary_peaks": {**pk, "philox_step_ceiling_flips_per_s": pk["philox_draws_per_s"] / 2.0,
                            "fp64_exp_log_step_ceiling_flips_per_s": fp64_step,
                            "achieved_flips_per_s": flips_per_s},
    }


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's path (oracle
    port) on every host thread, the same 400 problems per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_run(threads, threads)
    tot_p, tot_s, tot_f = 0.0, 0.0, 0.0
    for _ in range(args.steps):
        pps, fps, dt = cpu_run(CPU_SAMPLE_PROBLEMS, threads)
        tot_p += pps * dt
        tot_f += fps * dt
        tot_s += dt
    v = tot_p / tot_s
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": "samples/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32+f64",
        "data": "synthetic, seeded Philox",
        "config": {"workload": WORKLOAD_TAG, "l2": "n/a (host cores)"},
        "flips_per_s": tot_f / tot_s,
        "cpu_baseline": {"value": v, "unit": "samples/s", "cores": threads, "kind": "port",
                         "sample": f"all {CPU_SAMPLE_PROBLEMS} problems per step on {threads} threads (the "
                                   f"reference has no CPU path; its CUDA build needs Boost and HDF5)"},
        "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def profile_case(name: str):
    """Small fixed cases for ncu captures (not bench numbers): `main6x6` = 152
    problems of the workload (samples 0-37 x ivhc, one per SM) capped at 20
    outer iterations; `large16` = the large-lattice leg's 152 16x16 problems
    (512-thread teams) capped at 3 outer iterations; `batched` = the
    heterogeneous batched leg's 2000 problems capped at 3 outer iterations
    (three main-run launches side by side: 12x12, 10x10, and 4x4-8x8 teams).
    Each is solved twice (capture the second solve's main-run launches)."""
    import qec_pf_wang_landau_gb300 as wlg
    wlg.build()
    if name == "main6x6":
        probs = problems(0)[:152]
        cap = 20
    elif name == "large16":
        c = LARGE
        probs = [wlg.problem(16, 16, prob=c["prob"], error_class=cl, seed=c["seed"], sample=k, pre_walkers=128,
                             pre_intervals=128, pre_iterations=100 * 256, intervals=64, walkers_per_interval=8,
                             overlap=0.3, alpha=0.8, beta=1e-8, iterations=1000, exchange_every=10)
                 for k in range(c["samples"]) for cl in "ivhc"]
        cap = 3
    elif name == "batched":
        probs = batched_problems()
        cap = 3
    else:
        raise SystemExit(f"unknown profile case {name}")
    for p in probs:
        p.max_outer = cap
    ctx = wlg.Context(0)
    for _ in range(2):
        out = ctx.solve_raw(probs)
    st = ctx.stats()
    steps = sum(r.flips / (p.intervals * p.walkers_per_interval) for p, (r, _, _, _) in zip(probs, out))
    print(json.dumps({"case": name, "main_ms": st["main_ms"], "main_forms": st["main_forms"],
                      "walker_steps_per_problem": steps / len(probs)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--profile-case", default=None, help="run a small fixed case for a profiler and exit")
    ap.add_argument("--leg", default=None,
                    choices=["serving", "batched", "large", "c3_arms", "large_converged", "large_saturated", "peaks"],
                    help="run one extra leg alone and print it")
    ap.add_argument("--per-group", type=int, default=None, help="c3_arms: samples per group")
    ap.add_argument("--sides", type=int, nargs="*", default=None, help="c3_arms: lattice sides")
    ap.add_argument("--side", type=int, default=None, help="large_converged: lattice side")
    ap.add_argument("--samples", type=int, default=None, help="large_converged: samples per class")
    ap.add_argument("--beta", type=float, default=None, help="large_converged: final ln f")
    ap.add_argument("--classes", default=None, help="large_converged: error classes, e.g. ivhc")
    ap.add_argument("--no-extra", action="store_true", help="skip the serving and batched legs")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.leg is not None:
        import qec_pf_wang_landau_gb300 as wlg
        wlg.build()
        legs = {"serving": serving_run, "batched": batched_run, "large": large_run,
                "c3_arms": lambda: c3_arms_run(args.per_group, args.sides),
                "large_converged": lambda: large_converged_run(args.side, args.samples, args.beta, args.classes),
                "large_saturated": large_saturated_run,
                "peaks": lambda: wlg.measure_peaks(0)}
        print(json.dumps(r4({args.leg: legs[args.leg]()})), flush=True)
        return
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
