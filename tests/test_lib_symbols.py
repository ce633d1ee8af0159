"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol (no GPU calls)."""
import re
import os
import ctypes

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_symbols():
    """Every entry point declared in include/*.h."""
    inc = os.path.join(ROOT, "include")
    src = "".join(open(os.path.join(inc, f)).read() for f in sorted(os.listdir(inc)) if f.endswith(".h"))
    return sorted(set(re.findall(r"^(?:int|long long|const char\*)\s+(bte\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from boltzmann_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["bte_grid_create", "bte_solve_steady", "bte_qoi", "bte_lu_factor", "bte_lu_solve", "bte_engine_step",
              "bte1d_step_x", "bte1d_step_v", "bte1d_lmat"]:
        assert s in syms


def test_every_declared_symbol_is_exported(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_loads(lib):
    from boltzmann_gb300 import _lib
    l = _lib.load()
    assert l.bte_last_error() is not None


def test_argument_errors_without_gpu(lib):
    """Argument validation happens before any CUDA call."""
    from boltzmann_gb300 import _lib
    l = _lib.load()
    rc = l.bte_grid_create(None, None, None)
    assert rc == -1
    assert b"null" in l.bte_last_error()


def test_fvm_entry_points_refuse_bad_arguments(lib):
    """The FVM entry points check their arguments before any device work: null pointers,
    sizes out of range and a missing handle return BTE_ERR_ARG (no GPU is touched)."""
    import ctypes as C
    from boltzmann_gb300 import _lib
    l = _lib.load()
    dp = C.POINTER(C.c_double)
    h = C.c_void_p()
    null = dp()
    one = (C.c_double * 64)(*([1.0] * 64))
    ptrs = [C.cast(one, dp)] * 11
    assert l.bte_fvm_create(0, 4, 4, 4, 2, 2, 2, *([null] * 11), C.byref(h)) < 0
    assert b"null" in l.bte_fvm_last_error()
    assert l.bte_fvm_create(0, 4, 3, 4, 2, 2, 2, *ptrs, C.byref(h)) < 0        # odd ordinate count
    assert l.bte_fvm_create(0, 4, 4, 4, 5, 2, 2, *ptrs, C.byref(h)) < 0        # more diagonals than cells
    assert b"range" in l.bte_fvm_last_error()
    coef = _lib.FvmCoef(1e-3, 1e-3, 1e-7, 1.0, 1.0, 1.0)
    info = (C.c_double * 4)()
    assert l.bte_fvm_step(None, C.byref(coef), 1.0, 0, None, None, 1e-10, 1e-14, 30, 100, info, None) < 0
    assert l.bte_fvm_mvec(None, C.byref(coef), None, None, None, None) < 0
    assert l.bte_fvm_sl_step(None, C.byref(coef), None, None, None, None) < 0
    assert l.bte_fvm_set_collision_inverse(None, null, null) < 0
    assert l.bte_fvm_destroy(None) == 0
