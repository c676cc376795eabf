"""Shared test helpers: reference-layout Wang-Landau states built from the
oracle's pre-run, and device mirrors of them."""
from __future__ import annotations

import ctypes as C

import numpy as np

import oracle as O


def prerun_outputs(X, Y, boundary, prob, cls, seed, R, walkers, n_int_pre, n_iter):
    N = X * Y
    seen = np.zeros(R * (4 * N + 1), np.uint8)
    J = np.zeros(R * 2 * N, np.int8)
    flat = np.zeros(R * n_int_pre * N, np.int8)
    flag = np.zeros(R * n_int_pre, np.int32)
    en = np.zeros(R * n_int_pre, np.int32)
    O.lib().orc_prerun(X, Y, boundary, C.c_float(prob), cls.encode(), seed, R, walkers, n_int_pre, n_iter,
                       O.ptr(seen), O.ptr(J), O.ptr(flat), O.ptr(flag), O.ptr(en))
    return dict(X=X, Y=Y, boundary=boundary, R=R, seen=seen, J=J, found_lat=flat, found_flag=flag,
                found_energy=en, n_int_pre=n_int_pre)


def mainrun_state(pre, I, W, overlap):
    """file_io.cpp:558-659 + mainrun.cu:79-184: the arrays the main run starts from."""
    X, Y, R = pre["X"], pre["Y"], pre["R"]
    N = X * Y
    L = 4 * N + 1
    spectrum, off_spec, start, end = [], [], [], []
    for k in range(R):
        h = pre["seen"][k * L:(k + 1) * L]
        nz = np.nonzero(h == 1)[0]
        lo, hi = int(nz[0]), int(nz[-1])
        off_spec.append(len(spectrum))
        spectrum.extend(h[lo:hi + 1].tolist())
        s, e, _, _ = O.interval_results(-2 * N + lo, -2 * N + hi, I, W, overlap)
        start.extend(s.tolist())
        end.extend(e.tolist())
    off_hist, acc = [], 0
    for b in range(R * I):
        ln = end[b] - start[b] + 1
        for _ in range(W):
            off_hist.append(acc)
            acc += ln
    lat = np.zeros(R * I * W * N, np.int8)
    npre = pre["n_int_pre"]
    for k in range(R):
        found = sorted((int(pre["found_energy"][k * npre + q]), q) for q in range(npre)
                       if pre["found_flag"][k * npre + q])
        for bl in range(I):
            b = k * I + bl
            pick = next(q for (en, q) in found if start[b] <= en <= end[b])
            src = pre["found_lat"][(k * npre + pick) * N:(k * npre + pick + 1) * N]
            for w in range(W):
                t = b * W + w
                lat[t * N:(t + 1) * N] = src
    T = R * I * W
    off_lat = (np.arange(T, dtype=np.int32) * N).astype(np.int32)
    E = O.calc_energy(pre["boundary"], lat, pre["J"], off_lat, X, Y, T, I * W)
    st = dict(X=X, Y=Y, boundary=pre["boundary"], R=R, I=I, W=W, N=N,
              J=pre["J"].copy(), spectrum=np.array(spectrum, np.int8), off_spec=np.array(off_spec, np.int32),
              start=np.array(start, np.int32), end=np.array(end, np.int32), off_hist=np.array(off_hist, np.int32),
              lattice=lat, off_lat=off_lat, E=E, H=np.zeros(acc, np.uint64), logG=np.zeros(acc, np.float64),
              factor=np.full(T, np.e, np.float64), off_iter=np.zeros(T, np.uint64), cond=np.zeros(R * I, np.int8),
              cond_inter=np.zeros(R, np.int32), perm=(np.arange(T) % W).astype(np.int32),
              found=np.zeros(T, np.int32), newE=np.zeros(T, np.int32))
    for b in range(R * I):
        for w in range(W):
            assert st["start"][b] <= E[b * W + w] <= st["end"][b]
    return st


ARRAYS = ["J", "spectrum", "off_spec", "start", "end", "off_hist", "lattice", "off_lat", "E", "H", "logG", "factor",
          "off_iter", "cond", "cond_inter", "perm", "found", "newE"]


def copy_state(st):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}


# ------------------------------------------------------- oracle-side steps --

def o_wang_landau(st, n_iter, seed):
    p = O.ptr
    T = st["R"] * st["I"] * st["W"]
    return O.lib().orc_wang_landau(p(st["lattice"]), p(st["J"]), p(st["H"]), p(st["logG"]), p(st["factor"]),
                                   p(st["E"]), p(st["newE"]), p(st["off_iter"]), p(st["found"]), p(st["start"]),
                                   p(st["end"]), p(st["off_hist"]), p(st["off_lat"]), p(st["cond"]),
                                   p(st["spectrum"]), p(st["off_spec"]), p(st["cond_inter"]), st["X"], st["Y"],
                                   n_iter, T, st["I"], st["I"] * st["W"], seed, st["boundary"])


def o_check_histogram(st, alpha):
    p = O.ptr
    T = st["R"] * st["I"] * st["W"]
    O.lib().orc_check_histogram(p(st["H"]), p(st["factor"]), p(st["cond"]), p(st["off_hist"]), p(st["end"]),
                                p(st["start"]), p(st["spectrum"]), p(st["off_spec"]), p(st["cond_inter"]), alpha, T,
                                st["I"] * st["W"], st["I"])


def o_average(st):
    p = O.ptr
    O.lib().orc_average_log_g(p(st["logG"]), p(st["start"]), p(st["end"]), p(st["spectrum"]), p(st["off_spec"]),
                              p(st["cond"]), p(st["off_hist"]), p(st["cond_inter"]), st["R"], st["W"], st["I"])


def o_reset_finish(st, beta):
    p = O.ptr
    O.lib().orc_reset_cond(p(st["cond"]), p(st["factor"]), st["R"] * st["I"], beta, st["W"])
    O.lib().orc_check_finished(p(st["cond_inter"]), p(st["cond"]), st["I"], st["R"])


def o_exchange(st, even, seed, global_parity=0):
    p = O.ptr
    O.lib().orc_replica_exchange(p(st["off_lat"]), p(st["E"]), p(st["perm"]), p(st["off_iter"]), p(st["start"]),
                                 p(st["end"]), p(st["off_hist"]), p(st["cond_inter"]), p(st["logG"]), int(even), seed,
                                 st["I"], st["I"] * st["W"], st["R"] * st["I"], global_parity)


# ----------------------------------------------------------- device mirror --

class Dev:
    """Device copies of a state's arrays (torch tensors) and the engine calls on them."""

    def __init__(self, torch, st):
        self.torch = torch
        self.st = st
        self.t = {}
        for k in ARRAYS:
            a = st[k]
            if a.dtype == np.uint64:
                self.t[k] = torch.from_numpy(a.view(np.int64).copy()).cuda()
            else:
                self.t[k] = torch.from_numpy(a.copy()).cuda()

    def p(self, k):
        return C.c_void_p(self.t[k].data_ptr())

    def get(self, k):
        a = self.t[k].cpu().numpy()
        return a.view(np.uint64) if self.st[k].dtype == np.uint64 else a

    def snapshot(self):
        self.torch.cuda.synchronize()
        return {k: self.get(k) for k in ARRAYS}

    def wang_landau(self, n_iter, seed):
        import qec_pf_wang_landau_gb300 as wlg
        s = self.st
        T = s["R"] * s["I"] * s["W"]
        wlg.call("wlg_wang_landau", self.p("lattice"), self.p("J"), self.p("H"), self.p("logG"), self.p("factor"),
                 self.p("E"), self.p("newE"), self.p("off_iter"), self.p("found"), self.p("start"), self.p("end"),
                 self.p("off_hist"), self.p("off_lat"), self.p("cond"), self.p("spectrum"), self.p("off_spec"),
                 self.p("cond_inter"), s["X"], s["Y"], n_iter, T, s["I"], s["I"] * s["W"], seed, s["boundary"], None)

    def check_histogram(self, alpha):
        import qec_pf_wang_landau_gb300 as wlg
        s = self.st
        T = s["R"] * s["I"] * s["W"]
        wlg.call("wlg_check_histogram", self.p("H"), self.p("factor"), self.p("cond"), self.p("off_hist"),
                 self.p("end"), self.p("start"), self.p("spectrum"), self.p("off_spec"), self.p("cond_inter"), alpha,
                 T, s["I"] * s["W"], s["I"], None)

    def average(self):
        import qec_pf_wang_landau_gb300 as wlg
        s = self.st
        wlg.call("wlg_average_log_g", self.p("logG"), self.p("start"), self.p("end"), self.p("spectrum"),
                 self.p("off_spec"), self.p("cond"), self.p("off_hist"), self.p("cond_inter"), s["R"], s["W"], s["I"],
                 None)

    def reset_finish(self, beta):
        import qec_pf_wang_landau_gb300 as wlg
        s = self.st
        wlg.call("wlg_reset_cond", self.p("cond"), self.p("factor"), s["R"] * s["I"], beta, s["W"], None)
        wlg.call("wlg_check_finished", self.p("cond_inter"), self.p("cond"), s["I"], s["R"], None)

    def exchange(self, even, seed, global_parity=0):
        import qec_pf_wang_landau_gb300 as wlg
        s = self.st
        wlg.call("wlg_replica_exchange", self.p("off_lat"), self.p("E"), self.p("perm"), self.p("off_iter"),
                 self.p("start"), self.p("end"), self.p("off_hist"), self.p("cond_inter"), self.p("logG"), int(even),
                 seed, s["I"], s["I"] * s["W"], s["R"] * s["I"], global_parity, None)


def assert_state_equal(dev_snap, st, where=""):
    for k in ARRAYS:
        a, b = dev_snap[k], st[k]
        if not np.array_equal(a, b):
            bad = np.nonzero(a != b)[0]
            raise AssertionError(f"{where}: {k} differs at {bad[:8].tolist()} (gpu {a[bad[:4]].tolist()} vs "
                                 f"oracle {b[bad[:4]].tolist()}); {len(bad)} entries")
