"""The engine's pre-run -> main-run hand-off (wlg_handoff, host code) against
the reference's own hand-off (src/file_io.cpp:558-659 with src/interval.cpp)
recorded in tests/golden/reference_handoff.npz by
tests/golden/make_reference_handoff_golden.py: 80 seeded single-sample
problems, their pre-run outputs and what the reference made of them (E_min,
E_max, windows, each window's start lattice) or that it refused them.  Needs
only the built library, not the reference's sources."""
import os

import numpy as np


def test_handoff_matches_reference_golden():
    import qec_pf_wang_landau_gb300 as wlg
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_handoff.npz"))
    o = dict(seen=0, J=0, flag=0, lat=0, win=0, starts=0)
    refused = 0
    for c, (X, Y, boundary, prob, cls, seed, pre_w, pre_i, pre_n, I, W, ov) in enumerate(g["params"]):
        X, Y, boundary, seed, pre_w, pre_i, pre_n, I, W = (int(v) for v in (X, Y, boundary, seed, pre_w, pre_i, pre_n,
                                                                            I, W))
        N = X * Y
        seen = g["seen"][o["seen"]:o["seen"] + 4 * N + 1]
        J = g["J"][o["J"]:o["J"] + 2 * N]
        flag = g["flag"][o["flag"]:o["flag"] + pre_i]
        energy = g["energy"][o["flag"]:o["flag"] + pre_i]
        lat = g["lat"][o["lat"]:o["lat"] + pre_i * N]
        start, end = g["start"][o["win"]:o["win"] + I], g["end"][o["win"]:o["win"] + I]
        starts = g["starts"][o["starts"]:o["starts"] + I * N].reshape(I, N)
        o["seen"] += 4 * N + 1
        o["J"] += 2 * N
        o["flag"] += pre_i
        o["lat"] += pre_i * N
        o["win"] += I
        o["starts"] += I * N
        p = wlg.problem(X, Y, boundary=boundary, prob=float(prob), error_class=chr(int(cls)), seed=seed,
                        pre_walkers=pre_w, pre_intervals=pre_i, pre_iterations=pre_n, intervals=I,
                        walkers_per_interval=W, overlap=float(ov))
        (m,) = wlg.handoff([p], seen, J, flag, energy, lat)
        if not g["ok"][c]:
            assert m["status"] != 0, c
            refused += 1
            continue
        assert m["status"] == 0, (c, m["status"])
        assert (m["e_min"], m["e_max"]) == (int(g["e_min"][c]), int(g["e_max"][c])), c
        lo, hi = m["e_min"] + 2 * N, m["e_max"] + 2 * N
        assert np.array_equal(m["spectrum"][lo:hi + 1], seen[lo:hi + 1]) and not m["spectrum"][:lo].any()
        assert np.array_equal(m["start"], start) and np.array_equal(m["end"], end), c
        assert np.array_equal(m["lattices"], starts), c
    assert 0 < refused < len(g["ok"])


def test_handoff_rejects_missing_buffers():
    import ctypes as C
    import qec_pf_wang_landau_gb300 as wlg
    p = wlg.problem(4, 4)
    arr = (wlg.Problem * 1)(p)
    st = wlg.lib().wlg_handoff(C.cast(arr, C.c_void_p), 1, *([None] * 12))
    assert st == 1  # WLG_ERR_INVALID
    assert wlg.lib().wlg_handoff(None, 0, *([None] * 12)) == 0  # an empty batch
