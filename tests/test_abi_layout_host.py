"""The ctypes mirrors of the C-ABI structures (boltzmann_gb300/_lib.py) have the C layouts of
include/*.h: a small C program compiled with gcc against the headers prints each structure's
size and field offsets, and they must equal the ctypes ones (no GPU, no CUDA)."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

# (C type, ctypes class name in _lib, header)
STRUCTS = [("bte_grid_desc", "GridDesc", "bte_gb300.h"), ("bte_solve_opts", "SolveOpts", "bte_gb300.h"),
           ("bte_transient_opts", "TransientOpts", "bte_gb300.h"), ("bte_fvm_coef", "FvmCoef", "bte_fvm_gb300.h")]


@pytest.fixture(scope="module")
def c_layouts(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    from boltzmann_gb300 import _lib
    src = ["#include <stdio.h>", "#include <stddef.h>"]
    src += ['#include "%s"' % h for h in sorted({s[2] for s in STRUCTS})]
    src.append("int main(void) {")
    for ctype, pyname, _ in STRUCTS:
        src.append('  printf("%s size %%zu\\n", sizeof(%s));' % (ctype, ctype))
        for fname, _ in getattr(_lib, pyname)._fields_:
            src.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (ctype, fname, ctype, fname))
    src += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    c = d / "layout.c"
    c.write_text("\n".join(src) + "\n")
    exe = d / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    lay = {}
    for line in out:
        if line.strip():
            t, f, v = line.split()
            lay[(t, f)] = int(v)
    return lay


@pytest.mark.parametrize("ctype,pyname,header", STRUCTS)
def test_ctypes_structure_matches_c_layout(c_layouts, ctype, pyname, header):
    from boltzmann_gb300 import _lib
    cls = getattr(_lib, pyname)
    assert ctypes.sizeof(cls) == c_layouts[(ctype, "size")]
    for fname, _ in cls._fields_:
        assert getattr(cls, fname).offset == c_layouts[(ctype, fname)], (ctype, fname)
