"""Syndrome front-end on the CPU (host code of the engine library, no GPU):
frustrated plaquettes of bond patterns and patterns built from syndromes.

A pattern built from the syndrome of the true disorder differs from it by a
gauge transformation and possibly logical chains, so the four error classes
of both have the same partition functions up to a permutation; checked
here with the oracle's exact transfer-matrix counts."""
import numpy as np
import pytest

import oracle as O


@pytest.fixture(scope="module")
def wlg():
    import qec_pf_wang_landau_gb300 as m
    m.build()
    return m


def frustration_np(J, X, Y, boundary):
    N = X * Y
    R = J[:N].reshape(X, Y).astype(int)
    D = J[N:].reshape(X, Y).astype(int)
    prod = R * np.roll(R, -1, 0) * D * np.roll(D, -1, 1)
    if boundary == 1:
        prod = prod[:X - 1, :Y - 1]
    return (prod < 0).astype(np.uint8).ravel()


def with_class(J, X, Y, cls):
    J = J.copy()
    N = X * Y
    if cls in "hc":
        J[N:N + Y] *= -1
    if cls in "vc":
        J[0:N:Y] *= -1
    return J


@pytest.mark.parametrize("X,Y,boundary", [(4, 4, 0), (5, 3, 0), (4, 6, 1), (7, 5, 1), (2, 2, 0), (2, 3, 1)])
def test_frustration_and_round_trip(wlg, X, Y, boundary):
    rng = np.random.default_rng(X * 100 + Y * 10 + boundary)
    for _ in range(20):
        J = np.where(rng.random(2 * X * Y) < 0.3, -1, 1).astype(np.int8)
        S = wlg.frustration(X, Y, boundary, J)
        assert np.array_equal(S, frustration_np(J, X, Y, boundary))
        J2 = wlg.couplings_from_syndrome(X, Y, boundary, S)
        assert set(np.unique(J2)) <= {-1, 1}
        assert np.array_equal(wlg.frustration(X, Y, boundary, J2), S)
        # the class chains leave the syndrome alone
        for c in "hvc":
            assert np.array_equal(wlg.frustration(X, Y, boundary, with_class(J, X, Y, c)), S)


@pytest.mark.parametrize("boundary", [0, 1])
def test_any_syndrome_has_a_pattern(wlg, boundary):
    X, Y = 6, 5
    P = wlg.plaquettes(X, Y, boundary)
    rng = np.random.default_rng(7 + boundary)
    for _ in range(30):
        S = (rng.random(P) < 0.2).astype(np.uint8)
        if boundary == 0 and S.sum() % 2:
            S[0] ^= 1
        J = wlg.couplings_from_syndrome(X, Y, boundary, S)
        assert np.array_equal(wlg.frustration(X, Y, boundary, J), S)
    assert not wlg.couplings_from_syndrome(X, Y, boundary, np.zeros(P, np.uint8)).tolist().count(-1)


def test_invalid_syndromes_and_shapes(wlg):
    S = np.zeros(16, np.uint8)
    S[3] = 1  # one defect on a torus: no pattern
    with pytest.raises(wlg.WlgError) as e:
        wlg.couplings_from_syndrome(4, 4, 0, S)
    assert e.value.status == 1
    S[3] = 2
    S[5] = 1
    with pytest.raises(wlg.WlgError):
        wlg.couplings_from_syndrome(4, 4, 0, S)
    with pytest.raises(wlg.WlgError):
        wlg.frustration(1, 4, 0, np.ones(8, np.int8))
    with pytest.raises(wlg.WlgError):
        wlg.frustration(4, 4, 2, np.ones(32, np.int8))


@pytest.mark.parametrize("boundary", [0, 1])
def test_syndrome_pattern_has_the_same_class_partition_functions(wlg, boundary):
    """Classes of the syndrome's pattern are the true disorder's classes,
    permuted: the same four exact log Z at the Nishimori temperature."""
    X = Y = 5
    p = 0.1
    bn = 0.5 * np.log((1 - p) / p)
    for sample in range(4):
        J = O.init_interactions(X, Y, sample + 1, 99, p, "i")[sample * 2 * X * Y:]
        J2 = wlg.couplings_from_syndrome(X, Y, boundary, wlg.frustration(X, Y, boundary, J))

        def log_z(Jc):
            cnt = O.exact_counts(Jc, X, Y, boundary)
            E = np.nonzero(cnt)[0] - 2 * X * Y
            return np.logaddexp.reduce(np.log(cnt[E + 2 * X * Y]) - bn * E)

        a = np.sort([log_z(with_class(J, X, Y, c)) for c in "ivhc"])
        b = np.sort([log_z(with_class(J2, X, Y, c)) for c in "ivhc"])
        assert np.allclose(a, b, rtol=0, atol=1e-9)
