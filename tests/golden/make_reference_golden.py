"""Generates tests/golden/reference_host.npz: outputs of the reference's own
host code, compiled from its sources by oracle/ref_build.build_host()
(src/interval.cpp and src/result_handling.cpp, driven by oracle/ref_host.cpp).

* intervals: seeded random (e_min, e_max, num_intervals, walkers, overlap)
  tuples and what wl::interval_results makes of them (or that it throws);
* stitching: walker log g in the main run's dense per-window layout, from
  seeded synthetic curves (random lattice sizes, energy steps 2 and 4,
  unreachable energies, 1-3 walkers, 2-11 windows) and from the oracle's
  main run of a few small problems, with the (E, log g) pairs
  result_handling_stitched_histogram writes for them.

Run from the repository root where the reference sources exist:
    python tests/golden/make_reference_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "reference_host.npz")


def interval_cases(rng, n):
    rows, ok, starts, ends, offs, tot, ln = [], [], [], [], [0], [], []
    while len(rows) < n:
        N = int(rng.integers(4, 700))
        lo = -2 * N + 2 * int(rng.integers(0, N // 2 + 1))
        hi = 2 * N - 2 * int(rng.integers(0, N // 2 + 1))
        if hi <= lo:
            continue
        I = int(rng.integers(1, 70))
        W = int(rng.integers(1, 9))
        ov = float(np.float32(rng.choice([0.1, 0.25, 0.3, 0.5, 0.75, rng.random()])))
        r = O.ref_interval(lo, hi, I, W, ov)
        rows.append((lo, hi, I, W, ov))
        ok.append(r is not None)
        if r is not None:
            starts.extend(r[0].tolist())
            ends.extend(r[1].tolist())
            tot.append(r[2])
            ln.append(r[3])
        else:
            tot.append(0)
            ln.append(0)
        offs.append(len(starts))
    return dict(iv_params=np.array(rows, np.float64), iv_ok=np.array(ok, np.int8),
                iv_start=np.array(starts, np.int32), iv_end=np.array(ends, np.int32), iv_off=np.array(offs, np.int64),
                iv_total=np.array(tot, np.int64), iv_len=np.array(ln, np.int32))


def synthetic_windows(rng):
    while True:
        X, Y = int(rng.integers(2, 9)), int(rng.integers(2, 9))
        N = X * Y
        step = int(rng.choice([2, 4]))
        lo = -2 * N + step * int(rng.integers(0, N // 4 + 1))
        hi = 2 * N - step * int(rng.integers(0, N // 4 + 1))
        if hi - lo < 4 * step:
            continue
        I, W = int(rng.integers(2, 12)), int(rng.integers(1, 4))
        ov = float(np.float32(rng.choice([0.1, 0.25, 0.5, 0.75])))
        try:
            s, e, _, _ = O.interval_results(lo, hi, I, W, ov)
        except ValueError:
            continue
        E = np.arange(lo, hi + 1)
        base = np.log1p(np.maximum(0, (hi - E) * (E - lo))) * float(rng.uniform(0.1, 3.0))
        base = base + rng.normal(0, 0.05, len(E))
        reach = ((E - lo) % step == 0) & (rng.random(len(E)) > 0.05)
        parts = []
        for b in range(I):
            idx = np.arange(s[b], e[b] + 1) - lo
            for _ in range(W):
                seg = np.zeros(len(idx))
                v = base[idx] + rng.normal(0, 0.02, len(idx)) + float(rng.uniform(0, 50))
                seg[reach[idx]] = v[reach[idx]]
                parts.append(seg)
        yield np.concatenate(parts), s, e, I, W, X, Y


def oracle_windows():
    from tests.test_engine_gpu import oracle_run
    cfgs = [(4, 4, 0, 0.04, "i", 12345, 3, 32, 8, 2000, 10, 3, 0.25, 0.8, 0.001, 1000, 20, 1, 0),
            (5, 4, 1, 0.2, "h", 99, 3, 32, 9, 3000, 5, 2, 0.5, 0.8, 0.005, 400, 3, 1, 0),
            (5, 5, 1, 0.2, "i", 31337, 2, 64, 16, 3000, 7, 3, 0.25, 0.8, 0.01, 800, 2, 1, 1)]
    for c in cfgs:
        X, Y, R, I, W = c[0], c[1], c[6], c[10], c[11]
        r = oracle_run(*c)
        for k in range(R):
            s, e = r["start"][k * I:(k + 1) * I], r["end"][k * I:(k + 1) * I]
            a0 = r["off_hist"][k * I * W]
            yield r["logG"][a0:a0 + int(np.sum((e - s + 1) * W))], s, e, I, W, X, Y


def stitch_cases(rng, n_synth):
    meta, lgs, ss, es, Es, Gs = [], [], [], [], [], []
    pos = [0, 0, 0]

    def add(lg, s, e, I, W, X, Y):
        rb = O.stitch(lg, s, e, I, W, X, Y, 0)
        if rb[0] != 0:  # the reference dereferences an empty key list there
            return False
        rc, E, G = O.ref_stitch(lg, s, e, I, W, X, Y)
        meta.append((I, W, X, Y, pos[0], len(lg), pos[1], pos[2], len(E), rc))
        lgs.append(np.asarray(lg, np.float64))
        ss.append(np.asarray(s, np.int32))
        es.append(np.asarray(e, np.int32))
        Es.append(E)
        Gs.append(G)
        pos[0] += len(lg)
        pos[1] += I
        pos[2] += len(E)
        return True

    for case in oracle_windows():
        add(*case)
    gen = synthetic_windows(rng)
    made = 0
    while made < n_synth:
        made += add(*next(gen))
    return dict(st_meta=np.array(meta, np.int64), st_lg=np.concatenate(lgs), st_start=np.concatenate(ss),
                st_end=np.concatenate(es), st_E=np.concatenate(Es).astype(np.int32),
                st_G=np.concatenate(Gs).astype(np.float64))


def main():
    if O.reference_host() is None:
        sys.exit("reference sources not found: nothing generated")
    rng = np.random.default_rng(20261203)
    data = interval_cases(rng, 3000)
    data.update(stitch_cases(rng, 150))
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes;", len(data["iv_ok"]), "interval cases,", len(data["st_meta"]),
          "stitching cases")


if __name__ == "__main__":
    main()
