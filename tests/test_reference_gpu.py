"""The reference's own CUDA kernels (compiled unmodified from its wl.cu into
a cubin) driven in its prerun/mainrun order: a cross-check of the harness
against exact enumeration, and of this engine against the reference's
results at WL statistical tolerance (the reference's pre-run is not
deterministic, so bit parity with it is not defined)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _stitch(windows, starts, ends, X, Y):
    W = 1
    flat = np.concatenate(windows)
    E = np.zeros(4 * X * Y + 1, np.int32)
    G = np.zeros(4 * X * Y + 1)
    n = C.c_int(0)
    rc = O.lib().orc_stitch(O.ptr(np.ascontiguousarray(flat)), O.ptr(np.ascontiguousarray(starts)),
                            O.ptr(np.ascontiguousarray(ends)), len(windows), W, X, Y, O.ptr(E), O.ptr(G), len(E),
                            C.byref(n), 0)
    assert rc == 0
    return E[:n.value], G[:n.value]


@pytest.fixture(scope="module")
def ref(cuda):
    L = O.reference_harness()
    if L is None:
        pytest.skip("reference cubin not available on this machine")
    return L


def test_reference_kernels_match_exact_enumeration_4x4(ref):
    R, I = 3, 10
    out = O.reference_run(4, 4, 0, 0.04, "i", 12345, R, 32, 8, 1000, I, 3, 0.25, 0.8, 1e-3, 1000, 20)
    assert out["status"] == 0
    for k in range(R):
        E, G = _stitch(out["windows"][k * I:(k + 1) * I], out["start"][k * I:(k + 1) * I],
                       out["end"][k * I:(k + 1) * I], 4, 4)
        J = O.init_interactions(4, 4, R, 12345, 0.04, "i")[k * 32:(k + 1) * 32]
        cnt = O.exact_counts(J, 4, 4, 0)
        assert set(E.tolist()) == set((np.nonzero(cnt)[0] - 32).tolist())
        err = G - np.log(cnt[E + 32])
        assert np.sqrt(np.mean(err ** 2)) < 0.25


def test_engine_error_not_worse_than_reference_6x6(ref):
    """6x6 periodic, class v, the reference's flags (exchange off as in its loop):
    both log g curves against the exact transfer-matrix density of states; the
    engine's error must be of the reference's size or smaller."""
    import qec_pf_wang_landau_gb300 as wlg
    R, I = 4, 10
    out = O.reference_run(6, 6, 0, 0.04, "v", 777, R, 128, 32, 1000, I, 3, 0.25, 0.8, 1e-3, 1000, 20)
    assert out["status"] == 0
    probs = [wlg.problem(6, 6, prob=0.04, error_class="v", seed=777, sample=k, exchange_mode=0) for k in range(R)]
    mine = wlg.Context(0).solve(probs)
    J = O.init_interactions(6, 6, R, 777, 0.04, "v")
    e_ref, e_mine = [], []
    for k in range(R):
        E, G = _stitch(out["windows"][k * I:(k + 1) * I], out["start"][k * I:(k + 1) * I],
                       out["end"][k * I:(k + 1) * I], 6, 6)
        r, E2, G2 = mine[k]
        assert r.status == 0
        cnt = O.exact_counts(J[k * 72:(k + 1) * 72], 6, 6, 0)
        exact_E = set((np.nonzero(cnt)[0] - 72).tolist())
        assert set(E2.tolist()) == exact_E
        e_ref.append(np.sqrt(np.mean((G - np.log(cnt[E + 72])) ** 2)))
        e_mine.append(np.sqrt(np.mean((G2 - np.log(cnt[E2 + 72])) ** 2)))
    assert max(e_ref) < 1.0 and max(e_mine) < 1.0
    assert np.mean(e_mine) < 1.5 * np.mean(e_ref) + 0.1, (e_mine, e_ref)
