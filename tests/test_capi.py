"""CPU tests of the C ABI: the engine library loads and exports every entry
point include/wlg.h declares, status strings, and the Python mirror's
struct layouts (no GPU compute)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "wlg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wlg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def engine():
    import qec_pf_wang_landau_gb300 as wlg
    wlg.build()
    return wlg


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "wlg_wang_landau" in syms and "wlg_solve" in syms and len(syms) >= 20


def test_library_exports_every_declared_symbol(engine):
    L = engine.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol(engine):
    assert set(declared_symbols()) == set(engine.SIGNATURES)


def test_status_strings(engine):
    L = engine.lib()
    assert L.wlg_status_string(0) == b"ok"
    assert b"new energy" in L.wlg_status_string(3)
    assert L.wlg_status_string(999) == b"unknown status"
    assert engine.version().startswith("wlg-gb300")


def test_struct_layouts_match_c(engine, tmp_path):
    """Every field offset of the ctypes mirrors equals the C compiler's."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = ((engine.Problem, "wlg_problem"), (engine.Result, "wlg_result"), (engine.Stats, "wlg_stats"),
               (engine.ServerConfig, "wlg_server_config"), (engine.Decoded, "wlg_decoded"),
               (engine.ServerStats, "wlg_server_stats"))
    lines = []
    for cls, cname in structs:
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "wlg.h"\nint main(void){' + "".join(lines)
                   + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cls, cname in structs:
        assert int(got[cname]) == C.sizeof(cls)
        for f, _ in cls._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(cls, f).offset, f


def test_invalid_arguments_rejected_without_gpu(engine):
    L = engine.lib()
    # validation happens before any CUDA call
    assert L.wlg_init_interactions(None, 16, 1, 0, C.c_float(0.1), None) == 1
    assert L.wlg_calc_energy(2, None, None, None, None, 4, 4, 1, 1, None) == 1
    assert L.wlg_wang_landau(*([None] * 17), 4, 4, 10, 30, 7, 30, 1, 0, None) == 1  # walkers % intervals != 0
    out = C.c_void_p()
    assert L.wlg_context_create(-1, 0, C.byref(out)) == 1
    assert L.wlg_server_create(0, None, None) == 1
    assert L.wlg_server_submit(None, None, 0, None) == 1
    assert L.wlg_server_poll(None, None, 0, None, 0) == 1
    assert L.wlg_server_destroy(None) == 1
    assert L.wlg_context_set_stream(None, None) == 1
    assert L.wlg_solve(None, None, 0, None, None, None, 0) == 1


def test_server_without_a_device_fails_cleanly(engine):
    """Creating a server where no GPU is visible returns WLG_ERR_CUDA (2)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    out = C.c_void_p()
    assert engine.lib().wlg_server_create(0, None, C.byref(out)) == 2
    assert out.value is None
