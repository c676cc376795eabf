"""The C++ examples of the maintainers' integration guide (at the repository
root) compile against include/wlg.h, so the guide cannot drift from the
header (argument counts, types and order, struct field order in the
aggregate initialisers); its Python example names only what the binding
has.  CPU only (syntax check, nothing runs)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GUIDE = os.path.join(ROOT, "INTEGRATION.md")

# Names the examples take from the surrounding caller code (the reference's
# mainrun.cu buffers and options, a caller's lattice and request variables).
STUBS = """
struct AnyPtr { template <class T> operator T*() const { return nullptr; } };
struct Buf { AnyPtr data() const { return {}; } };
struct Options {
  int X = 4, Y = 4, num_iterations = 1000, num_intervals = 10, seed = 1, boundary = 0, num_interactions = 1,
      walker_per_interval = 3;
  double alpha = 0.8, beta = 1e-3;
};
"""
LOCALS = """
  Buf d_lattice, d_interactions, d_H, d_logG, d_factor, d_energy, d_newEnergies, d_offset_iter,
      d_foundNewEnergyFlag, d_start, d_end, d_offset_histogram, d_offset_lattice, d_cond,
      d_expected_energy_spectrum, d_offset_energy_spectrum, d_cond_interactions, d_max, d_indices;
  Options options;
  int total_walker = 30, walker_per_interactions = 30, total_intervals = 10;
  int X = 4, Y = 4, boundary = 0, seed = 1, R = 2, k = 0;
  float p = 0.04f;
  const unsigned char* syndrome = nullptr;
  wlg_server* srv = nullptr;
  wlg_problem req{};
  unsigned long long id = 0;
"""


def cpp_blocks():
    text = open(GUIDE).read()
    return re.findall(r"```cpp\n(.*?)```", text, re.S)


def test_guide_has_cpp_examples():
    assert len(cpp_blocks()) >= 4


def test_cpp_examples_compile_against_the_header(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    head = ["#include <cstddef>", "#include <stdexcept>", "#include <vector>", '#include "wlg.h"', STUBS]
    body = []
    for i, block in enumerate(cpp_blocks()):
        lines = block.splitlines()
        head += [ln for ln in lines if ln.startswith("#")]
        code = "\n".join(ln for ln in lines if not ln.startswith("#"))
        body.append(f"void example_{i}() {{\n{LOCALS}\n  {{\n{code}\n  }}\n}}\n")
    src = tmp_path / "examples.cpp"
    src.write_text("\n".join(head) + "\n" + "\n".join(body))
    r = subprocess.run([cxx, "-std=c++20", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_python_example_names_exist():
    """Every wlg.<name> the Python example uses exists in the binding, and the
    methods it calls exist on Context and Server."""
    import ast
    import qec_pf_wang_landau_gb300 as wlg
    text = open(GUIDE).read()
    (block,) = re.findall(r"```python\n(.*?)```", text, re.S)
    tree = ast.parse(block)
    for node in ast.walk(tree):
        if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name) and node.value.id == "wlg":
            assert hasattr(wlg, node.attr), node.attr
    for cls, methods in ((wlg.Context, ("solve", "set_stitching")), (wlg.Server, ("submit", "wait"))):
        for m in methods:
            assert callable(getattr(cls, m)), (cls.__name__, m)
