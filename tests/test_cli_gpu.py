"""The prerun/mainrun programs: the reference's flags, paths and file
layouts on the engine (bin/wlg_prerun, bin/wlg_mainrun).

The pre-run file must hold exactly the oracle's pre-run (visited energies,
couplings, stored lattices keyed by energy), and the main-run file exactly
the batch engine's stitched log g for the same problems with the
reference's exchange behaviour.
"""
import ctypes as C
import os
import subprocess
import time

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "qec_pf_wang_landau_gb300", "bin")
X, Y, R, SEED, P = 4, 4, 3, 12345, 0.04
PRE = ["-x", str(X), "-y", str(Y), "-p", str(P), "-n", "1000", "-w", "32", "-s", str(SEED), "-i", "8", "-e", "i",
       "-r", str(R), "-d", "7"]
MAIN = ["-x", str(X), "-y", str(Y), "-n", "1000", "-p", str(P), "-a", "0.8", "-b", "0.001", "-i", "10", "-w", "3",
        "-o", "0.25", "-s", str(SEED), "-e", "i", "-r", str(R), "-c", "20", "-d", "7", "-f", "3600"]
SUB = f"task_id_7/seed_{SEED}/periodic/prob_0.040000/X_{X}_Y_{Y}/error_class_i"


def run(prog, args, cwd):
    return subprocess.run([os.path.join(BIN, prog), *args], cwd=cwd, capture_output=True, text=True, timeout=600)


def oracle_prerun():
    N = X * Y
    seen = np.zeros(R * (4 * N + 1), np.uint8)
    J = np.zeros(R * 2 * N, np.int8)
    flat = np.zeros(R * 8 * N, np.int8)
    flag = np.zeros(R * 8, np.int32)
    en = np.zeros(R * 8, np.int32)
    O.lib().orc_prerun(X, Y, 0, C.c_float(P), b"i", SEED, R, 32, 8, 1000, O.ptr(seen), O.ptr(J), O.ptr(flat),
                       O.ptr(flag), O.ptr(en))
    return seen, J, flat, flag, en


def test_prerun_program_writes_the_oracle_prerun(cuda, tmp_path):
    import qec_pf_wang_landau_gb300 as wlg
    r = run("wlg_prerun", PRE, tmp_path)
    assert r.returncode == 0, r.stderr
    path = str(tmp_path / "init" / SUB / "prerun_results.h5")
    seen, J, flat, flag, en = oracle_prerun()
    N = X * Y
    assert wlg.h5_list(path)[0] == ["Histogram", "Interaction", "Lattice"]
    for k in range(R):
        h = wlg.h5_read(path, f"Histogram/{k}/Histogram")
        assert h.dtype == np.dtype("<u8") and np.array_equal(h, seen[k * (4 * N + 1):(k + 1) * (4 * N + 1)])
        assert np.array_equal(wlg.h5_read(path, f"Interaction/{k}/Interaction"), J[k * 2 * N:(k + 1) * 2 * N])
        want = {int(en[k * 8 + b]): flat[(k * 8 + b) * N:(k * 8 + b + 1) * N] for b in range(8) if flag[k * 8 + b]}
        groups, _ = wlg.h5_list(path, f"Lattice/{k}")
        assert sorted(int(g) for g in groups) == sorted(want)
        for e, lat in want.items():
            assert np.array_equal(wlg.h5_read(path, f"Lattice/{k}/{e}/Lattice"), lat)
    # the reference refuses to overwrite a pre-run file
    r2 = run("wlg_prerun", PRE, tmp_path)
    assert r2.returncode != 0 and "already exists" in r2.stderr


def batch_solve(wlg, xmode):
    probs = [wlg.problem(X, Y, prob=P, error_class="i", seed=SEED, sample=k, pre_walkers=32, pre_intervals=8,
                         pre_iterations=1000, intervals=10, walkers_per_interval=3, overlap=0.25, alpha=0.8,
                         beta=0.001, iterations=1000, exchange_every=20, exchange_mode=xmode, global_parity=1)
             for k in range(R)]
    return wlg.Context(0).solve(probs)


@pytest.mark.parametrize("xmode", [0, 1])
def test_mainrun_program_writes_the_engine_result(cuda, tmp_path, xmode):
    import qec_pf_wang_landau_gb300 as wlg
    assert run("wlg_prerun", PRE, tmp_path).returncode == 0
    r = run("wlg_mainrun", MAIN + ["--exchange-mode", str(xmode)], tmp_path)
    assert r.returncode == 0, r.stderr
    path = str(tmp_path / "results" / SUB / "mainrun_results.h5")
    ref = batch_solve(wlg, xmode)
    samples = sorted(int(g) for g in wlg.h5_list(path)[0])
    assert samples == [k for k, (res, _, _) in enumerate(ref) if res.status == 0]
    for k in samples:
        (stamp,), _ = wlg.h5_list(path, f"{k}/{SEED}")
        kv = wlg.h5_read(path, f"{k}/{SEED}/{stamp}/log_g")
        _, E, G = ref[k]
        assert np.array_equal(kv["Key"], E) and np.array_equal(kv["Value"], G)
        assert wlg.h5_attribute(path, f"{k}/{SEED}/{stamp}/log_g", "CodeVersion") == wlg.version()
    # a second run extends the file with a new timestamp group
    time.sleep(1.1)
    assert run("wlg_mainrun", MAIN + ["--exchange-mode", str(xmode)], tmp_path).returncode == 0
    for k in samples:
        assert len(wlg.h5_list(path, f"{k}/{SEED}")[0]) == 2


def test_mainrun_reads_a_prerun_file_in_libhdf5_default_structure(cuda, tmp_path):
    """The pre-run file rewritten in the structure libhdf5 writes by default
    (superblock 0, version-1 object headers, symbol-table groups; the
    reference's own prerun output) gives the same main-run file."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import h5v0
    import qec_pf_wang_landau_gb300 as wlg
    assert run("wlg_prerun", PRE, tmp_path).returncode == 0
    pre = str(tmp_path / "init" / SUB / "prerun_results.h5")

    def tree(prefix):
        groups, datasets = wlg.h5_list(pre, prefix)
        out = {g: tree(f"{prefix}/{g}") for g in groups}
        out.update({d: h5v0.Dataset(wlg.h5_read(pre, f"{prefix}/{d}")) for d in datasets})
        return out

    t = tree("")
    os.remove(pre)
    h5v0.write(pre, t)
    with open(pre, "rb") as f:
        assert f.read(9)[8] == 0  # superblock version 0
    r = run("wlg_mainrun", MAIN + ["--exchange-mode", "0"], tmp_path)
    assert r.returncode == 0, r.stderr
    path = str(tmp_path / "results" / SUB / "mainrun_results.h5")
    ref = batch_solve(wlg, 0)
    samples = sorted(int(g) for g in wlg.h5_list(path)[0])
    assert samples == [k for k, (res, _, _) in enumerate(ref) if res.status == 0]
    for k in samples:
        (stamp,), _ = wlg.h5_list(path, f"{k}/{SEED}")
        kv = wlg.h5_read(path, f"{k}/{SEED}/{stamp}/log_g")
        _, E, G = ref[k]
        assert np.array_equal(kv["Key"], E) and np.array_equal(kv["Value"], G)


def test_programs_on_an_open_lattice(cuda, tmp_path):
    """--boundary 1 on both programs: the files go under .../open/... (utils.cpp:88-128), the pre-run file
    holds the oracle's open-boundary pre-run, and the main-run file the batch engine's open-boundary log g."""
    import qec_pf_wang_landau_gb300 as wlg
    Xo, Yo = 5, 4
    pre = [a for a in PRE]
    main = [a for a in MAIN]
    for lst in (pre, main):
        lst[lst.index("-x") + 1], lst[lst.index("-y") + 1] = str(Xo), str(Yo)
        lst += ["--boundary", "1"]
    assert run("wlg_prerun", pre, tmp_path).returncode == 0
    sub = f"task_id_7/seed_{SEED}/open/prob_0.040000/X_{Xo}_Y_{Yo}/error_class_i"
    path = str(tmp_path / "init" / sub / "prerun_results.h5")
    N = Xo * Yo
    seen = np.zeros(R * (4 * N + 1), np.uint8)
    J = np.zeros(R * 2 * N, np.int8)
    flat = np.zeros(R * 8 * N, np.int8)
    flag = np.zeros(R * 8, np.int32)
    en = np.zeros(R * 8, np.int32)
    O.lib().orc_prerun(Xo, Yo, 1, C.c_float(P), b"i", SEED, R, 32, 8, 1000, O.ptr(seen), O.ptr(J), O.ptr(flat),
                       O.ptr(flag), O.ptr(en))
    for k in range(R):
        assert np.array_equal(wlg.h5_read(path, f"Histogram/{k}/Histogram"), seen[k * (4 * N + 1):(k + 1) * (4 * N + 1)])
        assert np.array_equal(wlg.h5_read(path, f"Interaction/{k}/Interaction"), J[k * 2 * N:(k + 1) * 2 * N])
    r = run("wlg_mainrun", main + ["--exchange-mode", "1"], tmp_path)
    assert r.returncode == 0, r.stderr
    out = str(tmp_path / "results" / sub / "mainrun_results.h5")
    probs = [wlg.problem(Xo, Yo, boundary=1, prob=P, error_class="i", seed=SEED, sample=k, pre_walkers=32,
                         pre_intervals=8, pre_iterations=1000, intervals=10, walkers_per_interval=3, overlap=0.25,
                         alpha=0.8, beta=0.001, iterations=1000, exchange_every=20, exchange_mode=1, global_parity=1)
             for k in range(R)]
    ref = wlg.Context(0).solve(probs)
    samples = sorted(int(g) for g in wlg.h5_list(out)[0])
    assert samples == [k for k, (res, _, _) in enumerate(ref) if res.status == 0] and samples
    for k in samples:
        (stamp,), _ = wlg.h5_list(out, f"{k}/{SEED}")
        kv = wlg.h5_read(out, f"{k}/{SEED}/{stamp}/log_g")
        _, E, G = ref[k]
        assert np.array_equal(kv["Key"], E) and np.array_equal(kv["Value"], G)


def test_mainrun_time_limit_and_flags(cuda, tmp_path):
    assert run("wlg_prerun", PRE, tmp_path).returncode == 0
    # -f 0: the run stops at the first check; no sample converges, nothing is written
    r = run("wlg_mainrun", [a if a != "3600" else "0" for a in MAIN], tmp_path)
    assert r.returncode == 0 and "Time limit" in r.stderr
    assert not (tmp_path / "results" / SUB / "mainrun_results.h5").exists()
    # help / version / missing required options: success without running
    assert run("wlg_mainrun", ["--help"], tmp_path).returncode == 0
    assert "WL mainrun version" in run("wlg_mainrun", ["-v"], tmp_path).stdout
    assert run("wlg_mainrun", ["-x", "4"], tmp_path).returncode == 0
    # no pre-run file for another seed: failure
    assert run("wlg_mainrun", [a if a != str(SEED) else "999" for a in MAIN], tmp_path).returncode != 0


@pytest.mark.parametrize("boundary", [0, 1])
def test_decode_program_equals_served_requests(cuda, tmp_path, boundary):
    """bin/wlg_decode: syndromes read from a file (comments and blank lines
    skipped), patterns built from them, served, one line per syndrome in
    input order: the same class log-probabilities as the same requests sent
    through the server's Python binding, and the most likely class."""
    import qec_pf_wang_landau_gb300 as wlg
    Xd, Yd, p = 5, 5, 0.08
    syn = []
    for k in range(5):
        Jk = O.init_interactions(Xd, Yd, k + 1, 777, p, "i")[k * 2 * Xd * Yd:(k + 1) * 2 * Xd * Yd]
        syn.append(wlg.frustration(Xd, Yd, boundary, Jk))
    f = tmp_path / "syndromes.txt"
    f.write_text("# five syndromes\n\n" + "\n".join("".join(str(int(b)) for b in s) for s in syn) + "\n")
    out = run("wlg_decode", ["-x", str(Xd), "-y", str(Yd), "-p", str(p), "--boundary", str(boundary), "-f", str(f),
                             "-b", "0.001", "-s", "3"], str(tmp_path))
    assert out.returncode == 0, out.stderr
    lines = [ln.split() for ln in out.stdout.strip().splitlines()]
    assert [int(ln[0]) for ln in lines] == list(range(5))
    reqs = [wlg.problem(Xd, Yd, boundary=boundary, prob=p, seed=3, sample=k, pre_walkers=128, pre_intervals=32,
                        pre_iterations=100 * Xd * Yd, intervals=4, walkers_per_interval=4, overlap=0.25, alpha=0.8,
                        beta=1e-3, iterations=1000, exchange_every=10, exchange_mode=1, global_parity=0)
            for k in range(5)]
    pats = [wlg.couplings_from_syndrome(Xd, Yd, boundary, s) for s in syn]
    with wlg.Server(0) as srv:
        ids = srv.submit(reqs, couplings=pats)
        got = srv.wait(ids, 300)
    for ln, i in zip(lines, ids):
        d = got[i]
        assert int(ln[1]) == d.status
        if d.status != 0:
            continue
        lp = [float(x) for x in ln[2:6]]
        assert np.allclose(lp, list(d.log_probs), rtol=1e-9, atol=1e-12)
        assert ln[6] == "ivhc"[int(np.argmax(d.log_probs))]
    bad = tmp_path / "bad.txt"
    bad.write_text("1" + "0" * (Xd * Yd - 1) + "\n")  # one defect
    out = run("wlg_decode", ["-x", str(Xd), "-y", str(Yd), "-p", str(p), "-f", str(bad)], str(tmp_path))
    if boundary == 0:
        assert out.returncode != 0 and "even" in out.stderr
