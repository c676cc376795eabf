"""Generates tests/golden/reference_handoff.npz: the reference's own
pre-run -> main-run hand-off (src/file_io.cpp:558-659 with src/interval.cpp,
chained as src/mainrun.cu:60-172 does, compiled from the reference's sources
by oracle/ref_build.build_host()) on the oracle's pre-run outputs of seeded
random single-sample problems: the inputs (the pre-run's visited energies,
couplings, stored lattices and their energies) and what the reference makes
of them, or that it refuses them (it throws when a window has no stored
lattice).

Run from the repository root where the reference sources exist:
    python tests/golden/make_reference_handoff_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from tests.helpers import prerun_outputs  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "reference_handoff.npz")


def main(n_cases=80):
    if O.reference_host() is None:
        sys.exit("reference sources not found: nothing generated")
    rng = np.random.default_rng(20261204)
    params, seen, J, flag, energy, lat, ok, lo, hi, start, end, starts = ([] for _ in range(12))
    while len(params) < n_cases:
        X, Y = int(rng.integers(3, 9)), int(rng.integers(3, 9))
        boundary = int(rng.integers(0, 2))
        prob = float(np.float32(rng.uniform(0.0, 0.3)))
        cls = "ivhc"[int(rng.integers(0, 4))]
        seed = int(rng.integers(-1000, 1000))
        pre_w, pre_i, pre_n = int(rng.integers(4, 65)), int(rng.integers(4, 33)), int(rng.integers(100, 3000))
        I, W = int(rng.integers(1, 15)), int(rng.integers(1, 5))
        ov = float(np.float32(rng.uniform(0.05, 0.9)))
        try:  # the reference's pre-run refuses coarse bins one energy wide (interval.cpp throws)
            O.interval_results(-2 * X * Y, 2 * X * Y, pre_i, 1, 1.0)
        except ValueError:
            continue
        pre = prerun_outputs(X, Y, boundary, prob, cls, seed, 1, pre_w, pre_i, pre_n)
        ref = O.ref_handoff(X, Y, 1, pre_i, I, W, ov, pre["seen"], pre["found_flag"], pre["found_energy"],
                            pre["found_lat"])
        N = X * Y
        params.append((X, Y, boundary, prob, ord(cls), seed, pre_w, pre_i, pre_n, I, W, ov))
        seen.append(pre["seen"])
        J.append(pre["J"])
        flag.append(pre["found_flag"])
        energy.append(pre["found_energy"])
        lat.append(pre["found_lat"])
        ok.append(ref is not None)
        if ref is not None:
            lo.append(int(ref["e_min"][0]))
            hi.append(int(ref["e_max"][0]))
            start.append(ref["start"])
            end.append(ref["end"])
            # every walker of a window starts from the same lattice: keep walker 0's
            starts.append(ref["lattices"][::W].reshape(-1))
        else:
            lo.append(0)
            hi.append(0)
            start.append(np.zeros(I, np.int32))
            end.append(np.zeros(I, np.int32))
            starts.append(np.zeros(I * N, np.int8))
    np.savez_compressed(OUT, params=np.array(params, np.float64), seen=np.concatenate(seen),
                        J=np.concatenate(J), flag=np.concatenate(flag), energy=np.concatenate(energy),
                        lat=np.concatenate(lat), ok=np.array(ok, np.int8), e_min=np.array(lo, np.int32),
                        e_max=np.array(hi, np.int32), start=np.concatenate(start), end=np.concatenate(end),
                        starts=np.concatenate(starts))
    print(OUT, os.path.getsize(OUT), "bytes;", n_cases, "cases,", sum(ok), "accepted by the reference")


if __name__ == "__main__":
    main()
