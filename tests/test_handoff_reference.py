"""The pre-run -> main-run hand-off against the reference's own code:
src/file_io.cpp:558-659 (spectrum trimming, start-lattice choice) and
src/interval.cpp, compiled from the reference's sources with a test-only
HDF5 declaration header (oracle/ref_host.cpp, oracle/h5stub) and chained as
src/mainrun.cu:60-172 chains them, against this engine's hand-off code
(wlg_handoff, host only), on the same pre-run outputs: E_min, E_max, the
trimmed spectrum, the windows and every walker's start lattice must be equal;
a sample the reference refuses (it throws) must be one the engine refuses.
Skipped where the reference sources are absent."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import prerun_outputs

pytestmark = pytest.mark.skipif(O.reference_host() is None, reason="reference sources not present")


def _sample(pre, k, N, pre_i):
    L = 4 * N + 1
    return (pre["seen"][k * L:(k + 1) * L], pre["found_flag"][k * pre_i:(k + 1) * pre_i],
            pre["found_energy"][k * pre_i:(k + 1) * pre_i], pre["found_lat"][k * pre_i * N:(k + 1) * pre_i * N])


def _compare(X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n, I, W, overlap):
    import qec_pf_wang_landau_gb300 as wlg
    N = X * Y
    pre = prerun_outputs(X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n)
    probs = [wlg.problem(X, Y, boundary=boundary, prob=prob, error_class=cls, seed=seed, sample=k, pre_walkers=pre_w,
                         pre_intervals=pre_i, pre_iterations=pre_n, intervals=I, walkers_per_interval=W,
                         overlap=overlap) for k in range(R)]
    mine = wlg.handoff(probs, pre["seen"], pre["J"], pre["found_flag"], pre["found_energy"], pre["found_lat"])
    refused = 0
    for k in range(R):
        ref = O.ref_handoff(X, Y, 1, pre_i, I, W, overlap, *_sample(pre, k, N, pre_i))
        m = mine[k]
        if ref is None:
            assert m["status"] != 0, (k, "the reference throws, the engine starts the main run")
            refused += 1
            continue
        assert m["status"] == 0, (k, m["status"])
        assert (m["e_min"], m["e_max"]) == (int(ref["e_min"][0]), int(ref["e_max"][0]))
        assert np.array_equal(m["spectrum"][m["e_min"] + 2 * N:m["e_max"] + 2 * N + 1], ref["spectrum"].view(np.uint8))
        assert not m["spectrum"][:m["e_min"] + 2 * N].any() and not m["spectrum"][m["e_max"] + 2 * N + 1:].any()
        assert np.array_equal(m["start"], ref["start"]) and np.array_equal(m["end"], ref["end"])
        for b in range(I):
            for w in range(W):
                assert np.array_equal(ref["lattices"][b * W + w], m["lattices"][b]), (k, b, w)
    if refused == 0:  # the whole run at once: per-sample offsets of the concatenated spectrum
        ref = O.ref_handoff(X, Y, R, pre_i, I, W, overlap, pre["seen"], pre["found_flag"], pre["found_energy"],
                            pre["found_lat"])
        assert ref is not None
        assert np.array_equal(ref["off_spec"], np.concatenate([[0], np.cumsum(ref["len_spec"])[:-1]]))
        assert np.array_equal(ref["start"], np.concatenate([m["start"] for m in mine]))
    return refused


@pytest.mark.parametrize("cfg", [
    (4, 4, 0, 0.04, "i", 12345, 3, 32, 8, 1000, 10, 3, 0.25),
    (6, 6, 0, 0.04, "c", 12345, 8, 128, 32, 1000, 10, 3, 0.25),
    (5, 7, 1, 0.1, "h", 9, 4, 64, 16, 2000, 6, 2, 0.4),
    (8, 8, 0, 0.12, "v", 77, 3, 128, 32, 6400, 12, 4, 0.3),
    (3, 9, 1, 0.3, "i", -5, 4, 16, 12, 3000, 4, 1, 0.1),
], ids=lambda c: f"{c[0]}x{c[1]}b{c[2]}{c[4]}")
def test_handoff_equals_reference(cfg):
    assert _compare(*cfg) == 0


def test_handoff_refusals_match_reference():
    """Few coarse pre-run bins (one stored lattice each at most) and many
    narrow windows: some samples have a window without a stored lattice;
    the reference throws for exactly those."""
    refused = 0
    for seed in range(6):
        refused += _compare(6, 6, seed % 2, 0.08, "ivhc"[seed % 4], 100 + seed, 6, 16, 16, 300, 14, 2, 0.8)
    assert 0 < refused < 36


def test_handoff_random_sweep():
    rng = np.random.default_rng(2468)
    for _ in range(40):
        X, Y = int(rng.integers(3, 9)), int(rng.integers(3, 9))
        _compare(X, Y, int(rng.integers(0, 2)), float(np.float32(rng.uniform(0.0, 0.3))), "ivhc"[int(rng.integers(0, 4))],
                 int(rng.integers(-1000, 1000)), int(rng.integers(1, 5)), int(rng.integers(4, 65)),
                 int(rng.integers(4, 33)), int(rng.integers(100, 3000)), int(rng.integers(1, 13)),
                 int(rng.integers(1, 5)), float(np.float32(rng.uniform(0.05, 0.6))))
