"""CPU tests against the reference's own host code compiled from its sources
(oracle/ref_host.cpp + src/interval.cpp + src/result_handling.cpp), fresh
random cases each run.  Skipped where the reference sources are absent; the
committed golden vectors (test_oracle_golden.py) cover those machines."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.skipif(O.reference_host() is None, reason="reference sources not present")


def test_interval_results_random_sweep():
    rng = np.random.default_rng()
    for _ in range(3000):
        N = int(rng.integers(4, 2000))
        lo = -2 * N + 2 * int(rng.integers(0, N // 2 + 1))
        hi = 2 * N - 2 * int(rng.integers(0, N // 2 + 1))
        if hi <= lo:
            continue
        I, W = int(rng.integers(1, 130)), int(rng.integers(1, 9))
        ov = float(np.float32(rng.random()))
        ref = O.ref_interval(lo, hi, I, W, ov)
        try:
            got = O.interval_results(lo, hi, I, W, ov)
        except ValueError:
            assert ref is None, (lo, hi, I, W, ov)
            continue
        assert ref is not None, (lo, hi, I, W, ov)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and got[2:] == ref[2:]


def test_stitching_random_sweep():
    from tests.golden.make_reference_golden import synthetic_windows
    gen = synthetic_windows(np.random.default_rng())
    checked = 0
    while checked < 300:
        lg, s, e, I, W, X, Y = next(gen)
        mine = O.stitch(lg, s, e, I, W, X, Y, 0)
        if mine[0] != 0:  # no stitch energy: the reference indexes an empty vector
            continue
        ref = O.ref_stitch(lg, s, e, I, W, X, Y)
        assert ref[0] == 0 and np.array_equal(mine[1], ref[1]) and np.array_equal(mine[2], ref[2])
        checked += 1
