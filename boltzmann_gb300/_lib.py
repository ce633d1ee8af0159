"""ctypes binding of `libbte_gb300.so` (the C ABI of include/bte_gb300.h).

There is no fallback: if the library is missing or fails to load, every entry point
raises. Build it with `python -m boltzmann_gb300._build` (or `__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbte_gb300.so")

PROC = {"ELASTIC": 0, "EXCITATION": 1, "IONIZATION": 2, "ATTACHMENT": 3}
PREC_FP64 = 0
PREC_MIXED = 1

OP = dict(KNOTS=0, MASS=1, MINV=2, ADV_RAW=3, COL_RAW=4, COL_GT_RAW=5, MASS_VEC=6, TEMP_VEC=7,
          MOBILITY=8, DIFFUSION=9, RATES=10, HL=11, GL=12, CC_A=13, CC_B=14, RADIAL_V3=15)

STATUS = {0: "converged", 1: "roundoff", 2: "max_iter", 3: "line_search", 4: "non_finite", 5: "singular"}

EXPORTED = ["bte_grid_create", "bte_grid_destroy", "bte_grid_info", "bte_grid_export", "bte_initialize",
            "bte_solve_steady", "bte_qoi", "bte_lu_factor", "bte_lu_solve", "bte_last_error",
            "bte_radial_components", "bte_stats_reset", "bte_stats", "bte_solve_info", "bte_lu_factor_ex",
            "bte_engine_create", "bte_engine_destroy", "bte_engine_admit", "bte_engine_step", "bte_engine_collect",
            "bte_engine_info", "bte_solve_transient", "bte1d_create", "bte1d_destroy", "bte1d_step_x", "bte1d_step_v", "bte1d_lmat", "bte1d_block_solve",
            "bte1d_ords_to_lm", "bte1d_lm_to_ords", "bte1d_launches", "bte1d_last_error", "bte1d_fim_matvec",
            "bte1d_step_fim",
            "bte_bidiag_solve", "bte_banded_tri_solve", "bte_banded_tri_mv", "bte_adv_be_sweep",
            "bte_bsr_upper_unit_solve", "bte_sweep_last_error", "bte_dgemm_nn", "bte_permute3",
            "bte_fvm_inflow_zero", "bte_fvm_create", "bte_fvm_destroy", "bte_fvm_set_collision_inverse",
            "bte_fvm_mvec", "bte_fvm_precond", "bte_fvm_step", "bte_fvm_launches", "bte_fvm_last_error",
            "bte_fvm_set_sl_grid", "bte_fvm_sl_advect", "bte_fvm_sl_step"]

STAT_FAMILIES = ["residual", "jacobian", "lu_factor", "lu_solve", "refine", "other", "lu_factor_fp64"]


class GridDesc(C.Structure):
    _fields_ = [
        ("n_sp", C.c_int), ("l_max", C.c_int), ("spline_qpts", C.c_int), ("vspace_ext", C.c_int),
        ("ee", C.c_int), ("ev_max", C.c_double), ("Te", C.c_double), ("mByM", C.c_double),
        ("n_processes", C.c_int), ("n_species", C.c_int),
        ("proc_type", C.POINTER(C.c_int)), ("proc_species", C.POINTER(C.c_int)),
        ("proc_threshold", C.POINTER(C.c_double)), ("proc_attach", C.POINTER(C.c_double)),
        ("sigma_offsets", C.POINTER(C.c_int)), ("sigma_energy", C.POINTER(C.c_double)),
        ("sigma_values", C.POINTER(C.c_double)), ("device", C.c_int), ("plain_knots", C.c_int),
    ]


class SolveOpts(C.Structure):
    _fields_ = [
        ("atol", C.c_double), ("rtol", C.c_double), ("max_iter", C.c_int),
        ("alpha_min", C.c_double), ("alpha_rho", C.c_double), ("line_search_c", C.c_double),
        ("ee", C.c_int), ("precision", C.c_int), ("refine", C.c_int), ("krylov", C.c_int), ("lu_kernel", C.c_int),
        ("lu64_kernel", C.c_int), ("reserved", C.c_int * 2),
    ]


class FvmCoef(C.Structure):
    """bte_fvm_coef (include/bte_fvm_gb300.h)."""
    _fields_ = [("dt", C.c_double), ("dtx", C.c_double), ("tau", C.c_double), ("kappa", C.c_double),
                ("cA", C.c_double), ("ax", C.c_double)]


class TransientOpts(C.Structure):
    _fields_ = [
        ("atol", C.c_double), ("rtol", C.c_double), ("max_iter", C.c_int), ("ee", C.c_int), ("precision", C.c_int),
        ("dt", C.c_double), ("cycles", C.c_double), ("efreq", C.c_double), ("reserved", C.c_int * 6),
    ]


_lib = None


def load() -> C.CDLL:
    """Load the library once; raise with a clear message when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libbte_gb300.so is not built (%s); run `python -m boltzmann_gb300._build`" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    vp, i32p = C.c_void_p, C.POINTER(C.c_int32)
    lib.bte_grid_create.argtypes = [C.POINTER(GridDesc), C.POINTER(C.c_void_p), vp]
    lib.bte_grid_destroy.argtypes = [vp]
    lib.bte_grid_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.bte_grid_export.argtypes = [vp, C.c_int, vp, C.c_size_t, vp]
    lib.bte_initialize.argtypes = [vp, C.c_int, vp, vp]
    lib.bte_solve_steady.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, C.POINTER(SolveOpts), vp]
    lib.bte_qoi.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp]
    lib.bte_lu_factor.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_longlong, vp, vp, vp]
    lib.bte_lu_solve.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_longlong, vp, vp, vp]
    lib.bte_lu_factor_ex.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_longlong, vp, vp, C.c_int, vp]
    lib.bte_last_error.restype = C.c_char_p
    lib.bte_stats_reset.argtypes = [C.c_int]
    lib.bte_solve_info.argtypes = [vp, C.c_int, vp, vp, vp]
    lib.bte_stats.argtypes = [C.POINTER(C.c_double), C.c_int]
    for name in EXPORTED:
        if not hasattr(lib, name):
            raise RuntimeError("libbte_gb300.so does not export %s" % name)
    lib.bte_engine_create.argtypes = [vp, C.c_int, C.c_int, C.POINTER(SolveOpts), C.POINTER(C.c_void_p)]
    lib.bte_engine_destroy.argtypes = [vp]
    lib.bte_engine_admit.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, i32p, vp]
    lib.bte_engine_step.argtypes = [vp, C.POINTER(C.c_int), i32p, vp]
    lib.bte_engine_collect.argtypes = [vp, C.c_int, i32p, vp, vp, vp, vp]
    lib.bte_engine_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_size_t)]
    dp = C.POINTER(C.c_double)
    lib.bte1d_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int] + [dp] * 9 + [C.c_int, C.POINTER(C.c_void_p)]
    lib.bte1d_destroy.argtypes = [vp]
    lib.bte1d_step_x.argtypes = [vp, C.c_double, vp, vp]
    lib.bte1d_step_v.argtypes = [vp, C.c_double, vp, vp, C.c_double, C.c_double, C.c_int, dp, vp]
    lib.bte1d_lmat.argtypes = [vp, C.c_double, vp, vp, vp, vp]
    lib.bte1d_block_solve.argtypes = [vp, C.c_double, vp, vp, vp, vp]
    lib.bte1d_fim_matvec.argtypes = [vp, C.c_double, vp, vp, vp, vp]
    lib.bte1d_step_fim.argtypes = [vp, C.c_double, vp, vp, C.c_double, C.c_double, C.c_int, C.c_int, dp, vp]
    lib.bte1d_ords_to_lm.argtypes = [vp, vp, vp, vp]
    lib.bte1d_lm_to_ords.argtypes = [vp, vp, vp, vp]
    lib.bte1d_launches.argtypes = [vp]
    lib.bte1d_launches.restype = C.c_longlong
    lib.bte1d_last_error.restype = C.c_char_p
    if hasattr(lib, "bte_initialize_noalloc"):
        lib.bte_initialize_noalloc.argtypes = [vp, C.c_int, vp, vp]
    if hasattr(lib, "bte_radial_components"):
        lib.bte_radial_components.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp]
    lib.bte_solve_transient.argtypes = [vp, C.c_int] + [vp] * 11 + [C.POINTER(TransientOpts), vp]
    ci = C.c_int
    lib.bte_bidiag_solve.argtypes = [ci, ci, vp, vp, vp, vp, ci, vp]
    lib.bte_banded_tri_solve.argtypes = [ci, ci, ci, vp, vp, vp, ci, vp]
    lib.bte_banded_tri_mv.argtypes = [ci, ci, ci, vp, vp, vp, ci, vp]
    lib.bte_adv_be_sweep.argtypes = [ci, vp, vp, vp, vp, C.c_double, vp, vp, ci, ci, ci, ci, vp]
    lib.bte_bsr_upper_unit_solve.argtypes = [ci, ci, ci, vp, vp, vp, vp, vp, vp]
    lib.bte_sweep_last_error.restype = C.c_char_p
    lib.bte_dgemm_nn.argtypes = [ci, ci, ci, vp, ci, vp, ci, vp, ci, vp]
    lib.bte_permute3.argtypes = [ci, ci, ci, ci, ci, ci, vp, vp, vp]
    lib.bte_fvm_inflow_zero.argtypes = [ci, ci, ci, vp, vp, vp]
    lib.bte_fvm_create.argtypes = [ci] * 7 + [dp] * 11 + [C.POINTER(vp)]
    lib.bte_fvm_destroy.argtypes = [vp]
    lib.bte_fvm_set_collision_inverse.argtypes = [vp, dp, dp]
    lib.bte_fvm_mvec.argtypes = [vp, C.POINTER(FvmCoef), vp, vp, vp, vp]
    lib.bte_fvm_precond.argtypes = [vp, C.c_double, C.c_double, C.c_double, vp, vp, vp, vp]
    lib.bte_fvm_step.argtypes = [vp, C.POINTER(FvmCoef), C.c_double, ci, vp, vp, C.c_double, C.c_double, ci, ci, dp, vp]
    lib.bte_fvm_set_sl_grid.argtypes = [vp, dp, C.c_double, C.c_double]
    lib.bte_fvm_sl_advect.argtypes = [vp, C.POINTER(FvmCoef), vp, vp, vp, vp]
    lib.bte_fvm_sl_step.argtypes = [vp, C.POINTER(FvmCoef), vp, vp, vp, vp]
    lib.bte_fvm_launches.argtypes = [vp]
    lib.bte_fvm_launches.restype = C.c_longlong
    lib.bte_fvm_last_error.restype = C.c_char_p
    _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        msg = load().bte_last_error().decode(errors="replace")
        raise RuntimeError("%s failed (code %d): %s" % (what, rc, msg))


def stats_reset(timing: bool) -> None:
    check(load().bte_stats_reset(int(timing)), "bte_stats_reset")


def stats() -> dict:
    """Kernel launches and per-family (launches, device ms, algorithmic flops, bytes)."""
    nb = 2 + 4 * len(STAT_FAMILIES) + 5
    buf = (C.c_double * nb)()
    check(load().bte_stats(buf, nb), "bte_stats")
    out = {"launches": int(buf[0])}
    for i, f in enumerate(STAT_FAMILIES):
        out[f] = dict(launches=int(buf[1 + 4 * i]), ms=buf[2 + 4 * i], flops=buf[3 + 4 * i], bytes=buf[4 + 4 * i])
    out["fp64_fallback_points"] = int(buf[1 + 4 * len(STAT_FAMILIES)])
    out["fp64_fallback_reasons"] = {k: int(buf[2 + 4 * len(STAT_FAMILIES) + i]) for i, k in
                                    enumerate(["max_iter", "line_search", "non_finite", "singular", "refinement"])}
    return out


def ptr(t) -> C.c_void_p:
    """Device pointer of a CUDA tensor (null for None)."""
    return C.c_void_p(0 if t is None else t.data_ptr())
