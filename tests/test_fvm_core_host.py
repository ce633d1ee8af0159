"""The shared core of the finite-volume fully implicit step (boltzmann_gb300/csrc/fvm_core.h),
compiled for the host through tests/host/fvm_harness.cpp: its operator, its op-split
preconditioner (closed-form collision inverse) and its GMRES against the reference's own
rhs_mvec, preconditioner and step (tests/golden/fvm_implicit_reference.npz), on the
product's host set-up and step coefficients (boltzmann_gb300.bte_1d3v_fvm.fvm_setup,
step_coefficients) from the fixture's parameter table."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from boltzmann_gb300 import bte_1d3v_fvm as P

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "boltzmann_gb300", "csrc")
GOLDEN = os.path.join(HERE, "golden", "fvm_implicit_reference.npz")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    so = str(tmp_path_factory.mktemp("fvm") / "fvm_harness.so")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC,
                        os.path.join(HERE, "host", "fvm_harness.cpp"), "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return C.CDLL(so)


@pytest.fixture(scope="module")
def case(synthetic_xs):
    """The product's host set-up and step coefficients from the fixture's parameter table."""
    from helpers import FVM_IMPLICIT_PARAMS
    g = dict(np.load(GOLDEN))
    st = P.fvm_setup(dict(FVM_IMPLICIT_PARAMS, collisions=synthetic_xs))
    for k in ("vr", "vt", "x"):
        np.testing.assert_allclose(st.grid_info[k], g[k], rtol=0, atol=1e-14 * np.abs(g[k]).max())
    p = st.params
    dt = float(g["dt"])
    c6 = np.array(P.step_coefficients(p, st.vth, dt, dt))
    np.testing.assert_allclose(c6, [dt, dt, float(g["tau"]), float(g["n0"]) * float(g["np0"]),
                                    float(g["qe"]) / float(g["me"]) / float(g["vth"]),
                                    float(g["vth"]) * float(g["tau"]) / float(g["L"])], rtol=1e-14)
    dinv, H = st.collisions.inverse_factors(dt * c6[2] * c6[3])
    return dict(g=g, p=[p.pvr, p.pvt, p.px], bands=st.bands, coll=st.collisions, dinv=dinv, H=H, c6=c6,
                cE=c6[2] * c6[4], ax=c6[5])


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


class _Args:
    """Keeps the marshalled arrays alive for one call."""

    def __init__(self, case):
        g = case["g"]
        self.keep = []
        self.dims = (C.c_int * 6)(int(g["Nr"]), int(g["Nvt"]), int(g["Nx"]), case["p"][0] + 1, case["p"][1] + 1,
                                  case["p"][2] + 1)
        bl = [case["bands"][k] for k in ("vr_diag_l2r", "vr_diag_r2l", "vt_diag_l2r", "vt_diag_r2l", "x_diag_l2r",
                                         "x_diag_r2l")]
        self.bands = (C.POINTER(C.c_double) * 6)(*[self.p(b) for b in bl])
        coll = case["coll"]
        self.common = [self.dims, self.p(g["vr"]), self.p(g["vt"]), self.p(coll.w), self.p(coll.loss),
                       self.p(coll.gain), self.bands]

    def p(self, a):
        arr, ptr = _d(a)
        self.keep.append(arr)
        return ptr


def test_operator_matches_the_reference(harness, case):
    g = case["g"]
    a = _Args(case)
    Y = np.zeros_like(g["u"])
    harness.fvm_host_mvec(*a.common, a.p(case["c6"]), a.p(g["E"]), a.p(g["u"]), Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - g["Au"])) <= 1e-12 * np.max(np.abs(g["Au"]))


def test_preconditioner_matches_the_reference_op_split_step(harness, case):
    g = case["g"]
    a = _Args(case)
    Y = np.zeros_like(g["u"])
    harness.fvm_host_precond(*a.common, a.p(case["dinv"]), a.p(case["H"]), C.c_double(case["cE"]),
                             C.c_double(case["ax"]), C.c_double(float(g["dt"])), a.p(g["E"]), a.p(g["u"]),
                             Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - g["Mu"])) <= 1e-12 * np.max(np.abs(g["Mu"]))


def test_preconditioner_with_half_step_sweeps_matches_the_oracle(harness, case):
    """gmres_pc_vr = 0.5: the reference's preconditioner takes the three sweeps (v_r, v_theta, x)
    over alpha dt while the collision solve keeps dt (bte_1d3v_solver.py:1819-1860). The core's
    preconditioner with hstep = 0.5 dt and the full-step collision factors against the oracle's
    op-split step at alpha = 0.5 (the oracle is pinned to the reference's step at alpha = 1),
    and it differs from the full-step preconditioner."""
    from oracle import bte1d_fvm_oracle as F
    g = case["g"]
    gs = dict(np.load(os.path.join(HERE, "golden", "fvm_reference.npz")))
    a = _Args(case)
    dt = float(g["dt"])
    Y = {}
    for alpha in (0.5, 1.0):
        y = np.zeros_like(g["u"])
        harness.fvm_host_precond(*a.common, a.p(case["dinv"]), a.p(case["H"]), C.c_double(case["cE"]),
                                 C.c_double(case["ax"]), C.c_double(alpha * dt), a.p(g["E"]), a.p(g["u"]),
                                 y.ctypes.data_as(C.POINTER(C.c_double)))
        Y[alpha] = y
    ref = F.op_split_step(gs, g["E"], np.asarray(g["u"]).reshape(-1, int(gs["Nx"])), dt, alpha=0.5).reshape(-1)
    assert np.max(np.abs(Y[0.5].reshape(-1) - ref)) <= 1e-12 * np.max(np.abs(ref))
    assert np.max(np.abs(Y[0.5] - Y[1.0])) > 1e-6 * np.max(np.abs(Y[1.0]))


@pytest.mark.parametrize("restart,pc_mode,alpha", [(30, 0, 1.0), (4, 0, 1.0), (30, 1, 1.0), (4, 1, 1.0), (30, 2, 1.0),
                                                   (30, 0, 0.5)])
def test_gmres_step_matches_the_reference(harness, case, restart, pc_mode, alpha):
    """The step to rtol 1e-12, the preconditioner on the right, on the left and none (also with
    a short restart, so that restarts happen, and with the preconditioner's step scaled by
    gmres_pc_vr = 0.5), against the reference's GMRES result."""
    g = case["g"]
    a = _Args(case)
    V = np.ascontiguousarray(g["v0"], dtype=np.float64).copy()
    info = (C.c_double * 4)()
    harness.fvm_host_step.restype = C.c_int
    rc = harness.fvm_host_step(*a.common, a.p(case["dinv"]), a.p(case["H"]), a.p(case["c6"]), C.c_double(alpha),
                               C.c_int(pc_mode), a.p(g["E"]), V.ctypes.data_as(C.POINTER(C.c_double)), C.c_double(float(g["rtol"])),
                               C.c_double(float(g["atol"])), C.c_int(restart), C.c_int(400), info)
    assert rc == 0
    assert info[3] == 0.0, list(info)
    assert 0 < info[0] <= 400
    ref = g["step"]
    assert np.max(np.abs(V - ref)) <= 1e-10 * np.max(np.abs(ref))


def test_semi_lagrangian_advection_matches_the_reference(harness):
    """step_adv_vx_sl: the departure points, the padded grid and the trilinear interpolation of
    the shared core against the reference's own interpolation (SciPy interpn on its CPU path)."""
    g = dict(np.load(os.path.join(HERE, "golden", "fvm_sl_reference.npz")))
    dims = (C.c_int * 3)(int(g["Nr"]), int(g["Nvt"]), int(g["Nx"]))
    keep = [np.ascontiguousarray(g[k], dtype=np.float64) for k in ("vr", "vt", "x", "E", "v0")]
    dt, tau, vth = float(g["dt"]), float(g["tau"]), float(g["vth"])
    cX = dt * tau * vth / float(g["L"])
    cE = dt * tau * float(g["qe"]) / float(g["me"]) / vth
    Y = np.zeros_like(keep[4])
    harness.fvm_host_sl(dims, *[_d(a)[1] for a in keep[:3]], C.c_double(float(g["kdomain"][0])),
                        C.c_double(float(g["kdomain"][1])), C.c_double(cX), C.c_double(cE), _d(keep[3])[1],
                        _d(keep[4])[1], Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - g["v_sl"])) <= 1e-13 * np.max(np.abs(g["v_sl"]))
    assert (Y == 0.0).any()          # departure points outside the domain (inflow)


def test_semi_lagrangian_step_matches_the_reference(harness, synthetic_xs):
    """The step: the shared core's advection, then the product's closed-form collision inverse
    built from the fixture's parameter table, against the reference's PmatC v_sl."""
    from helpers import FVM_SL_PARAMS
    g = dict(np.load(os.path.join(HERE, "golden", "fvm_sl_reference.npz")))
    st = P.fvm_setup(dict(FVM_SL_PARAMS, collisions=synthetic_xs))
    p = st.params
    dt = float(p.dt)
    c6 = P.step_coefficients(p, st.vth, dt, dt)
    dims = (C.c_int * 3)(len(st.vr), len(st.vt), len(st.x))
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (st.vr, st.vt, st.x, g["E"], g["v0"])]
    Y = np.zeros_like(keep[4])
    harness.fvm_host_sl(dims, *[_d(a)[1] for a in keep[:3]], C.c_double(0.0), C.c_double(st.vmax),
                        C.c_double(dt * c6[5]), C.c_double(dt * c6[2] * c6[4]), _d(keep[3])[1], _d(keep[4])[1],
                        Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - g["v_sl"])) <= 1e-13 * np.max(np.abs(g["v_sl"]))
    y = st.collisions.inverse_dense(dt * c6[2] * c6[3]) @ Y
    assert np.max(np.abs(y - g["step"])) <= 1e-12 * np.max(np.abs(g["step"]))


@pytest.mark.parametrize("pc_left", [1, 0])
def test_gmres_on_the_reference_test_system(harness, pc_left):
    """The solver alone on the system of the reference's own GMRES test (test_gmres.py:12-22):
    A = I + 0.1 U(0,1) (n = 1000), the Jacobi preconditioner, restart 20, rtol 1e-12, against a
    dense solve; both preconditioner sides (the reference's test runs the left one)."""
    rng = np.random.default_rng(0)
    n = 1000
    A = np.eye(n) + 1e-1 * rng.random((n, n))
    minv = 1.0 / np.diag(A)
    b = rng.random(n)
    x = np.zeros(n)
    info = (C.c_double * 4)()
    harness.gmres_host_dense.restype = C.c_int
    rc = harness.gmres_host_dense(C.c_int(n), _d(A)[1], _d(minv)[1], _d(b)[1], x.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_int(20), C.c_double(1e-12), C.c_double(1e-20), C.c_int(500), C.c_int(pc_left),
                                  info)
    assert rc == 0 and info[3] == 0.0, list(info)
    assert np.linalg.norm(b - A @ x) <= 1e-12 * np.linalg.norm(b) * 1.0001
    xs = np.linalg.solve(A, b)
    assert np.max(np.abs(x - xs)) <= 1e-9 * np.max(np.abs(xs))


@pytest.mark.parametrize("Nr_sp,Nvt,Nx,p,seed", [(6, 4, 7, 1, 1), (9, 6, 9, 3, 2), (7, 10, 5, 2, 3), (8, 8, 11, 3, 4)])
def test_core_against_the_oracle_on_other_grids(harness, synthetic_xs, Nr_sp, Nvt, Nx, p, seed):
    """The operator, the preconditioner and the semi-Lagrangian advection of the shared core
    against the oracle's restatements on grids and stencil orders the fixtures do not cover
    (orders 1 and 3, odd and even sizes), with a field of both signs."""
    from oracle import bte1d_fvm_oracle as F
    from boltzmann_gb300.bte_1d3v import ordinates
    from boltzmann_gb300.lxcat import read_cross_section_data
    rng = np.random.default_rng(seed)
    vr, vr_qw, vmax = P.radial_cells(80.0, 4.0, Nr_sp, 3, 3)
    vt, vt_qw = ordinates(Nvt)
    x = P.x_points(Nx)
    vth = P.thermal_velocity(4.0)
    procs = list(read_cross_section_data(synthetic_xs).values())
    coll = P.FvmCollisions(*P.fvm_collisions(procs, vr, vt_qw, vth, vmax), 2.0 * np.pi * vt_qw)
    bands = P.fvm_bands(P.fvm_upwind_operators(vr, vt, x, p, p, p, vmax), p, p, p)
    Nr = len(vr)
    dt, tau, L, kappa = 2e-3, 7.4e-8, 1.27e-2, 3.2e22
    cA = 1.602176634e-19 / 9.1093837139e-31 / vth
    ax = vth * tau / L
    E = 4e4 * rng.standard_normal(Nx)
    u = rng.standard_normal((Nr * Nvt, Nx))
    g = dict(Nr=Nr, Nvt=Nvt, Nx=Nx, pvr=p, pvt=p, px=p, tau=tau, qe=1.602176634e-19, me=9.1093837139e-31,
             vth=vth, L=L, vr=vr, vt=vt, n0=kappa, np0=1.0, op_col_en=coll.dense(),
             PmatC=coll.inverse_dense(dt * tau * kappa), **bands)
    case = dict(g=dict(g, Nr=np.array(Nr), Nvt=np.array(Nvt), Nx=np.array(Nx)), p=[p, p, p], bands=bands, coll=coll)
    a = _Args(case)
    # operator
    Ep, En = F.adv_v_fvm(vr, vt, p, p, vmax)
    xs = F.x_shift_bands(vr, vt, x, p, ax, dt)
    ref = F.implicit_matvec(g, cA * Ep, cA * En, xs, E, u, dt)
    Y = np.zeros_like(u)
    harness.fvm_host_mvec(*a.common, a.p([dt, dt, tau, kappa, cA, ax]), a.p(E), a.p(u),
                          Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - ref)) <= 1e-12 * np.max(np.abs(ref))
    # preconditioner
    dinv, H = coll.inverse_factors(dt * tau * kappa)
    ref = F.op_split_step(g, E, u, dt)
    harness.fvm_host_precond(*a.common, a.p(dinv), a.p(H), C.c_double(tau * cA), C.c_double(ax), C.c_double(dt),
                             a.p(E), a.p(u), Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - ref)) <= 1e-11 * np.max(np.abs(ref))
    # semi-Lagrangian advection at a step and field that move the departure points by a fraction
    # of a cell to a few cells in x and in v
    dts, Es = 5e-3, 0.1 * E
    ref = F.sl_advect(u, vr, vt, x, Es, dts, tau, vth, L, g["qe"], g["me"], 0.0, vmax)
    assert 0.0 < np.mean(ref == 0.0) < 0.5
    dims = (C.c_int * 3)(Nr, Nvt, Nx)
    harness.fvm_host_sl(dims, a.p(vr), a.p(vt), a.p(x), C.c_double(0.0), C.c_double(vmax), C.c_double(dts * ax),
                        C.c_double(dts * tau * cA), a.p(Es), a.p(u), Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_zero_step_is_the_identity(harness, case):
    """Edge case: at dt = 0 every departure point is its own grid point, so the semi-Lagrangian
    advection returns its input (to the rounding of sqrt(v^2) and acos(cos(theta)) in the
    departure point), and the fully implicit operator is the identity."""
    g = case["g"]
    a = _Args(case)
    u = np.ascontiguousarray(g["u"].reshape(-1, int(g["Nx"])))
    dims = (C.c_int * 3)(int(g["Nr"]), int(g["Nvt"]), int(g["Nx"]))
    Y = np.zeros_like(u)
    harness.fvm_host_sl(dims, a.p(g["vr"]), a.p(g["vt"]), a.p(g["x"]), C.c_double(0.0), C.c_double(float(g["domain"][1])),
                        C.c_double(0.0), C.c_double(0.0), a.p(g["E"]), a.p(u), Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.max(np.abs(Y - u)) <= 1e-14 * np.max(np.abs(u))
    c6 = np.array(case["c6"])
    c6[0] = c6[1] = 0.0
    harness.fvm_host_mvec(*a.common, a.p(c6), a.p(g["E"]), a.p(u), Y.ctypes.data_as(C.POINTER(C.c_double)))
    assert np.array_equal(Y, u)


def test_operator_column_by_column(harness, case):
    """Matrix-free against assembled, the reference's own matvec test pattern
    (test_bte_1d_matvec.py): the shared core's rhs_mvec on every unit vector equals the
    oracle's operator, column by column."""
    from oracle import bte1d_fvm_oracle as F
    g = case["g"]
    Nr, Nvt, Nx = int(g["Nr"]), int(g["Nvt"]), int(g["Nx"])
    n = Nr * Nvt * Nx
    c6 = case["c6"]
    Ep, En = F.adv_v_fvm(g["vr"], g["vt"], *case["p"][:2], float(g["domain"][1]))
    xs = F.x_shift_bands(g["vr"], g["vt"], g["x"], case["p"][2], float(c6[5]), float(c6[1]))
    go = dict(g, op_col_en=case["coll"].dense(), n0=float(c6[3]), np0=1.0)
    a = _Args(case)
    pc, pE = a.p(c6), a.p(g["E"])
    e = np.zeros((n // Nx, Nx))
    col = np.zeros_like(e)
    worst = 0.0
    for k in range(n):
        e.reshape(-1)[k] = 1.0
        harness.fvm_host_mvec(*a.common, pc, pE, e.ctypes.data_as(C.POINTER(C.c_double)),
                              col.ctypes.data_as(C.POINTER(C.c_double)))
        ref = F.implicit_matvec(go, c6[4] * Ep, c6[4] * En, xs, g["E"], e, float(c6[0]))
        worst = max(worst, np.max(np.abs(col - ref)) / max(np.max(np.abs(ref)), 1e-300))
        e.reshape(-1)[k] = 0.0
    assert worst <= 1e-12, worst


def test_preconditioner_column_by_column(harness, case):
    """The op-split preconditioner (closed-form collision inverse and sweeps) on unit vectors
    equals the oracle's op-split step with the dense PmatC, column by column: 300 seeded
    columns plus both ends of the first and the last x line."""
    from oracle import bte1d_fvm_oracle as F
    g = case["g"]
    Nx = int(g["Nx"])
    n = int(g["Nr"]) * int(g["Nvt"]) * Nx
    dt = float(case["c6"][0])
    go = dict(g, PmatC=case["coll"].inverse_dense(dt * case["c6"][2] * case["c6"][3]), **case["bands"])
    a = _Args(case)
    pd, pH, pE = a.p(case["dinv"]), a.p(case["H"]), a.p(g["E"])
    e = np.zeros((n // Nx, Nx))
    col = np.zeros_like(e)
    worst = 0.0
    cols = set(np.random.default_rng(6).choice(n, 300, replace=False).tolist())
    cols |= {0, Nx - 1, n - Nx, n - 1}
    for k in sorted(cols):
        e.reshape(-1)[k] = 1.0
        harness.fvm_host_precond(*a.common, pd, pH, C.c_double(case["cE"]), C.c_double(case["ax"]), C.c_double(dt), pE,
                                 e.ctypes.data_as(C.POINTER(C.c_double)), col.ctypes.data_as(C.POINTER(C.c_double)))
        ref = F.op_split_step(go, g["E"], e, dt)
        worst = max(worst, np.max(np.abs(col - ref)) / max(np.max(np.abs(ref)), 1e-300))
        e.reshape(-1)[k] = 0.0
    assert worst <= 1e-11, worst
