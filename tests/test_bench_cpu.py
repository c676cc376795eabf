"""bench.py on CPU: every leg the JSON line reports exists, and the synthetic
workloads follow their specifications (no GPU needed to build them)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_legs_exist():
    import bench
    for name in ("run_ours", "run_reference", "serving_run", "batched_run", "large_run", "accuracy", "plain_run",
                 "reference_cuda_run", "cpu_run", "profile_case", "reduce_over_ranks"):
        assert callable(getattr(bench, name)), name


def test_headline_workload():
    import bench
    probs = bench.problems(0)
    assert len(probs) == 400
    assert {(p.X, p.Y, p.boundary, round(p.prob, 6)) for p in probs} == {(6, 6, 0, 0.04)}
    assert sorted({p.sample for p in probs}) == list(range(100))
    assert {(p.intervals, p.walkers_per_interval, p.iterations, p.exchange_every) for p in probs} == {(10, 3, 1000, 20)}


def test_serving_workload_is_poisson_at_200_per_second():
    import bench
    arrivals, reqs = bench.serving_requests()
    assert 120 < len(reqs) < 280  # 200 expected in 1 s
    gaps = np.diff([0.0] + arrivals)
    assert abs(gaps.mean() - 1 / 200) < 0.0015
    assert {r.X for r in reqs} <= set(range(4, 17)) and all(r.X == r.Y for r in reqs)
    assert all(0.02 <= r.prob <= 0.12 and r.beta == 1e-6 and r.boundary == 0 for r in reqs)


def test_batched_workload():
    import bench
    probs = bench.batched_problems()
    assert len(probs) == 2000
    assert {p.X for p in probs} == {4, 6, 8, 10, 12}
    assert {p.boundary for p in probs} == {0, 1}
    assert {p.error_class for p in probs} == {b"i", b"v", b"h", b"c"}
    assert all(8 <= p.intervals <= 32 and p.walkers_per_interval == 4 and p.beta == 1e-6 for p in probs)


def test_accuracy_scores_exact_curves_as_exact():
    """The accuracy leg on curves that are the exact log g themselves (shifted
    by a constant, as a normalisation error would): zero RMS after the
    shift's own size, energy sets exact, every class decision equal to the
    exact one; a failed problem leaves its sample out of the decisions."""
    import types
    import bench
    import oracle as O
    w = bench.WORKLOAD
    N = w["X"] * w["Y"]
    out = []
    Js = {c: O.init_interactions(w["X"], w["Y"], w["samples"], w["seed"], w["prob"], c) for c in w["classes"]}
    for k in range(w["samples"]):
        for c in w["classes"]:
            cnt = O.exact_counts(Js[c][k * 2 * N:(k + 1) * 2 * N], w["X"], w["Y"], w["boundary"])
            E = (np.nonzero(cnt)[0] - 2 * N).astype(np.int32)
            out.append((types.SimpleNamespace(status=0), E, np.log(cnt[E + 2 * N]) + 1e-3))
    out[5] = (types.SimpleNamespace(status=3), np.zeros(0, np.int32), np.zeros(0))  # sample 1, class v
    acc = bench.accuracy({"engine": out, "engine_x0": out[:5] + out[5:]}, None)
    assert acc["engine_sets_exact"] and abs(acc["rms"]["engine"] - 1e-3) < 1e-9
    assert acc["rms"]["engine_x0"] == acc["rms"]["engine"] and "reference_cuda" not in acc["rms"]
    d = acc["class_decisions_equal_exact"]
    assert acc["samples"] == 100 and d["engine"] == 99 and d["engine_x0"] == 99 and d["reference_cuda"] == 0
    assert sum(acc["exact_class_counts"].values()) == 100


def test_r4_shortens_numbers_only():
    import bench
    assert bench.r4({"a": 1234.5678, "b": [0.000123456, 3, "x"], "c": float("nan")}) == \
        {"a": 1235.0, "b": [0.0001235, 3, "x"], "c": None}


def test_batched_accuracy_scores_every_side_against_exact():
    """The batched leg's scoring on curves that are the exact log g of each
    problem (one periodic and one open per side up to 10, one open 12x12,
    which the transfer matrix walks in one pass): zero error, energy sets
    exact, at most the stated number of curves per side, and a problem that
    did not converge is skipped."""
    import types
    import bench
    import oracle as O
    probs, out = [], []
    for L in (4, 6, 8, 10, 12):
        for boundary in ((0, 1) if L <= 10 else (1,)):
            p = types.SimpleNamespace(X=L, Y=L, boundary=boundary, sample=3, seed=77, prob=0.08,
                                      error_class=b"h")
            N = L * L
            J = O.init_interactions(L, L, p.sample + 1, p.seed, p.prob, "h")[p.sample * 2 * N:]
            cnt = O.exact_counts(J, L, L, boundary)
            E = (np.nonzero(cnt)[0] - 2 * N).astype(np.int32)
            probs.append(p)
            out.append((types.SimpleNamespace(status=0), E, np.log(cnt[E + 2 * N])))
    probs.insert(0, probs[0])
    out.insert(0, (types.SimpleNamespace(status=3), np.zeros(0, np.int32), np.zeros(0)))
    acc = bench.batched_accuracy(probs, out)
    assert set(acc) == {f"{L}x{L}" for L in (4, 6, 8, 10, 12)}
    for L in (4, 6, 8, 10, 12):
        a = acc[f"{L}x{L}"]
        assert a["curves"] == min(2 if L <= 10 else 1, bench.BATCHED_ACCURACY_PER_SIDE[L])
        assert a["energy_sets_exact"]
        assert a["rms_mean"] < 1e-12 and a["max_abs"] < 1e-12


def test_headline_line_fits_the_kept_tail():
    """The headline line, with every key at a worst-case width, stays within
    the last 1500 characters of output that a run's record keeps (newline
    included)."""
    import json
    import bench
    legs = {"batched": {"value": 97.71234, "status_counts": {"0": 1990, "3": 10}, "critical_path_ms": 17920.123,
                        "main_ms": 19850.456, "accuracy": {f"{L}x{L}": {"rms_mean": 0.0712345} for L in (4, 6, 8, 10, 12)}},
            "large": {"workload": "w", "16x16": {"flips_per_s": 80480000000.0}, "24x24": {"flips_per_s": 6.785e10}},
            "large_saturated": {"workload": "w", "16x16": {"reference_over_engine": 60.59123, "plain_over_engine": 4.12123},
                                "24x24": {"reference_over_engine": 46.77123, "plain_over_engine": 3.60823}},
            "large_converged": {k: {"value": 0.2047123, "rms_vs_reference": 0.1193456}
                                for k in ("engine", "engine_x0", "plain", "reference_cuda")},
            "serving": {"retired_ok": 165, "requests": 165, "requests_readmitted": 20, "p50_ms": 5023.123,
                        "p99_ms": 63920.123}}
    line = {"metric": bench.METRIC, "value": 6065.123, "unit": "samples/s", "n_gpus": 1, "steps": 20, "warmup": 5,
            "ms_per_step": 65.95123, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32+f64", "data": "synthetic, seeded Philox",
            "config": {"workload": "6x6 pbc p.04 100x4cls pre128/32/1000 I10 W3 o.25 a.8 lnf1e-3 n1000 c20",
                       "l2": "flushed", "teams_per_cta": {"f2/t32": 4}},
            "e2e": {"value": 5927.123, "unit": "samples/s", "h2d_bytes_per_step": 237140, "d2h_bytes_per_step": 1000880},
            "gpu_launches": 100, "roofline": {"bound": "hbm", "achieved": 529.123, "peak": 6677.0, "unit": "GB/s",
                                              "frac": 0.0792512, "traffic": 797440, "peak_kind": "measured",
                                              "smem_frac": 0.01319123},
            "flips_per_s": 15560000000.0, "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"]},
            "cpu_baseline": {"value": 182.5123, "unit": "samples/s", "cores": 72, "kind": "port",
                             "sample": "96 problems"},
            "arms": {"plain": 237.4123, "x0": 7105.123, "ref": 138.4123, "x0/ref": 51.33123, "v/plain": 25.54123},
            "accuracy": {"rms": {"eng": 0.17871, "x0": 0.1841, "ref": 0.1731},
                         "cls_ok": {"eng": 100, "x0": 99, "ref": 98}, "of": 100, "sets_ok": True},
            "legs": bench.legs_summary(legs)}
    assert len(json.dumps(bench.r4(line))) + 1 <= 1490


def test_critical_path_names_the_longest_chain_and_the_last_problem():
    """critical_path on made-up main-run times: the longest span, the problem
    that ends last (a late starter with a shorter span), the latest start per
    side, the most problems running at once; problems without a main run
    (start -1) are left out."""
    import types
    import bench

    class Ctx:
        def main_times(self):
            return (np.array([0.0, 0.0, 3000.0, -1.0, 100.0]), np.array([9000.0, 2000.0, 11000.0, -1.0, 600.0]))

    probs = [types.SimpleNamespace(X=x, Y=x, boundary=0, intervals=8) for x in (12, 10, 10, 8, 12)]
    out = [(types.SimpleNamespace(outer_iterations=n),) for n in (900, 200, 700, 0, 50)]
    cp = bench.critical_path(Ctx(), probs, out)
    assert cp["critical_path_ms"] == 9000.0 and cp["critical_problem"]["side"] == 12
    assert cp["critical_problem"]["outer_iterations"] == 900 and cp["critical_problem"]["us_per_outer"] == 1e4
    assert cp["last_problem"] == {"side": 10, "start_ms": 3000.0, "span_ms": 8000.0, "outer_iterations": 700}
    assert cp["start_ms_max_by_side"] == {"10x10": 3000.0, "12x12": 100.0}
    assert cp["last_end_ms"] == 11000.0 and cp["concurrent_peak"] == 3


def test_a_failing_leg_is_reported_not_raised():
    import bench

    def broken():
        raise RuntimeError("no device")
    legs = {"batched": bench.run_leg(broken), "serving": {"retired_ok": 3, "requests": 3, "requests_readmitted": 0,
                                                        "p99_ms": 1500.0}}
    assert legs["batched"] == {"error": "RuntimeError: no device"}
    import time
    late = bench.run_leg(lambda: {"value": 1.0}, time.perf_counter() - bench.LEG_BUDGET_S - 1)
    assert late["error"].startswith("skipped")
    assert bench.run_leg(lambda: {"value": 1.0}, time.perf_counter()) == {"value": 1.0}
    assert bench.legs_summary(legs) == {"failed": ["batched"], "serving": {"ok": "3/3", "readm": 0, "p99_s": 1.5}}
