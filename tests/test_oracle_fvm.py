"""The FVM 1D3V op-split oracle and the sweeps' band storage against the reference's own
set-up and step (tests/golden/fvm_reference.npz, made by tests/golden/make_golden_fvm.py)."""
import os

import numpy as np
import pytest

from oracle import bte1d_fvm_oracle as F
from oracle import sweeps_oracle as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fvm_reference.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


def _band_part(D, nd, lower):
    """D restricted to its first nd diagonals below (lower) or above the main one."""
    N = D.shape[0]
    i, j = np.indices((N, N))
    k = (i - j) if lower else (j - i)
    return np.where((k >= 0) & (k < nd), D, 0.0)


def test_band_storage_is_the_reference_upwind_operators(g):
    """The sweeps read D[i][i-k] at band[k][i-k] (lower) and D[i][i+k] at band[k][i+k] (upper):
    the reference's band arrays, read that way, are its dense upwind matrices (v_theta's after
    the diag(sin theta) factor init() applies, bte_1d3v_solver.py:1449-1450)."""
    sin_vt = np.diag(np.sin(g["vt"]))
    for band_l, band_r, DL, DR, nd in (
            (g["vr_diag_l2r"], g["vr_diag_r2l"], g["Dvr_LtoR"], g["Dvr_RtoL"], int(g["pvr"]) + 1),
            (g["vt_diag_l2r"], g["vt_diag_r2l"], sin_vt @ g["Dvt_LtoR"], sin_vt @ g["Dvt_RtoL"], int(g["pvt"]) + 1),
            (g["x_diag_l2r"], g["x_diag_r2l"], g["Dx_LtoR"], g["Dx_RtoL"], int(g["px"]) + 1)):
        np.testing.assert_allclose(S.band_by_column_to_dense(band_l, True), _band_part(DL, nd, True), rtol=0, atol=1e-12 * np.abs(DL).max())
        np.testing.assert_allclose(S.band_by_column_to_dense(band_r, False), _band_part(DR, nd, False), rtol=0, atol=1e-12 * np.abs(DR).max())
        # the upwind stencils fit in the stored band
        assert np.abs(DL - _band_part(DL, nd, True)).max() <= 1e-12 * np.abs(DL).max()
        assert np.abs(DR - _band_part(DR, nd, False)).max() <= 1e-12 * np.abs(DR).max()


def test_op_split_step_matches_the_reference(g):
    y = F.op_split_step(g, g["E"], g["v0"], float(g["dt"]))
    ref = g["step"]
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_collision_operator_and_inverse_on_the_fvm_grid(g, synthetic_xs):
    """The oracle's FVM grid, strong-form collision operator and PmatC against the reference's
    (same cross sections: the synthetic LXCat file the fixture was made from)."""
    from oracle import bte_oracle as O
    from oracle import bte1d_oracle as O1
    Nr = int(g["Nr"])
    ops = O.Operators(O.processes_from_lxcat(synthetic_xs), 80.0, 4.0, 8, 0, ee=False, snap=False)
    vr, vr_qw = F.fvm_vr_grid(ops.basis, int(g["spline_qpts"]))
    np.testing.assert_allclose(vr, g["vr"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(vr_qw, g["vr_qw"], rtol=1e-13, atol=0)
    vt, vt_qw = O1.gl_vt(int(g["Nvt"]))
    np.testing.assert_allclose(vt, g["vt"], rtol=1e-14, atol=0)
    C = F.collision_op_fvm(O.processes_from_lxcat(synthetic_xs), vr, vr_qw, vt, vt_qw, float(g["vth"]),
                           float(g["domain"][1]), O.C_GAMMA)
    ref = g["op_col_en"]
    assert np.max(np.abs(C - ref)) <= 1e-12 * np.max(np.abs(ref))
    P = F.collision_inverse(ref, float(g["dt"]), float(g["tau"]), float(g["n0"]), float(g["np0"]))
    assert np.max(np.abs(P - g["PmatC"])) <= 1e-10 * np.max(np.abs(g["PmatC"]))
    assert len(vr) == Nr


def test_upwind_operators_and_bands(g):
    """The oracle's upwind derivative operators (own Lagrange weights) and the six band arrays
    against the reference's (mesh.upwinded_dx / upwinded_dvt through init())."""
    p = {k: int(g[k]) for k in ("pvr", "pvt", "px")}
    for D, x, sw, dirn, theta in ((g["Dx_LtoR"], g["x"], p["px"] + 1, "L", False),
                                  (g["Dx_RtoL"], g["x"], p["px"] + 1, "R", False),
                                  (g["Dvt_LtoR"], g["vt"], p["pvt"] + 1, "L", True),
                                  (g["Dvt_RtoL"], g["vt"], p["pvt"] + 1, "R", True)):
        mine = (F.upwind_d1_theta if theta else F.upwind_d1)(np.asarray(x), sw, dirn)
        # the captured arrays carry init()'s inflow-row zeroing
        if dirn == "L":
            mine[0, :] = 0.0
        else:
            mine[-1, :] = 0.0
        assert np.max(np.abs(mine - D)) <= 1e-9 * np.max(np.abs(D))
    bands = F.fvm_upwind_bands(g["vr"], g["vt"], g["x"], p["pvr"], p["pvt"], p["px"], float(g["domain"][1]))
    for k, b in bands.items():
        ref = g[k]
        assert np.max(np.abs(b - ref)) <= 1e-9 * np.max(np.abs(ref)), k


GOLDEN_IMPLICIT = os.path.join(os.path.dirname(__file__), "golden", "fvm_implicit_reference.npz")


@pytest.fixture(scope="module")
def gi(g):
    """The fully implicit fixture (same grid as the op-split one), with the op-split fixture's
    collision operator."""
    d = dict(np.load(GOLDEN_IMPLICIT))
    for k in ("vr", "vt", "x"):
        assert np.array_equal(d[k], g[k])
    d["op_col_en"] = g["op_col_en"]
    return d


def _implicit_ops(gi):
    s = float(gi["qe"]) / float(gi["me"]) / float(gi["vth"])
    Ep, En = F.adv_v_fvm(gi["vr"], gi["vt"], int(gi["pvr"]), int(gi["pvt"]), float(gi["domain"][1]))
    ax = float(gi["vth"]) * float(gi["tau"]) / float(gi["L"])
    xs = F.x_shift_bands(gi["vr"], gi["vt"], gi["x"], int(gi["px"]), ax, float(gi["dt"]))
    return s * Ep, s * En, xs


def test_implicit_operators_match_the_reference(gi):
    Ep, En, xs = _implicit_ops(gi)
    for mine, ref in ((Ep, gi["adv_v_Ep"]), (En, gi["adv_v_En"])):
        assert np.max(np.abs(mine - ref)) <= 1e-13 * np.max(np.abs(ref))
    assert np.max(np.abs(xs - gi["x_shift_diag"])) <= 1e-13 * np.max(np.abs(gi["x_shift_diag"]))


def test_implicit_matvec_rhs_and_step_match_the_reference(gi):
    """rhs_mvec on a seeded vector, the right-hand side, and the step (a direct solve against
    the reference's GMRES to rtol 1e-12; the field has both signs)."""
    Ep, En, xs = _implicit_ops(gi)
    assert (gi["E"] < 0).any() and (gi["E"] > 0).any()
    dt = float(gi["dt"])
    Au = F.implicit_matvec(gi, Ep, En, xs, gi["E"], gi["u"], dt).reshape(-1)
    assert np.max(np.abs(Au - gi["Au"])) <= 1e-13 * np.max(np.abs(gi["Au"]))
    assert np.array_equal(F.implicit_rhs(gi, gi["v0"]).reshape(-1), gi["brhs"])
    y = F.implicit_step(gi, Ep, En, xs, gi["E"], gi["v0"], dt)
    assert np.max(np.abs(y - gi["step"])) <= 1e-10 * np.max(np.abs(gi["step"]))


def test_implicit_preconditioner_is_the_op_split_step(g, gi):
    Mu = F.op_split_step(g, gi["E"], gi["u"].reshape(-1, int(g["Nx"])), float(g["dt"]))
    assert np.max(np.abs(Mu.reshape(-1) - gi["Mu"])) <= 1e-13 * np.max(np.abs(gi["Mu"]))


def test_semi_lagrangian_step_matches_the_reference():
    """The oracle's explicit trilinear interpolation at the departure points against the
    reference's own step_adv_vx_sl (SciPy interpn) and step (PmatC v_sl)."""
    gs = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "fvm_sl_reference.npz")))
    v_sl = F.sl_advect(gs["v0"], gs["vr"], gs["vt"], gs["x"], gs["E"], float(gs["dt"]), float(gs["tau"]),
                       float(gs["vth"]), float(gs["L"]), float(gs["qe"]), float(gs["me"]), float(gs["kdomain"][0]),
                       float(gs["kdomain"][1]))
    assert np.max(np.abs(v_sl - gs["v_sl"])) <= 1e-14 * np.max(np.abs(gs["v_sl"]))
    assert np.max(np.abs(gs["PmatC"] @ v_sl - gs["step"])) <= 1e-14 * np.max(np.abs(gs["step"]))


@pytest.mark.parametrize("p", [1, 3])
def test_upwind_operators_at_other_orders(p):
    """The oracle's bands, v-space advection matrices and x-shift bands against the reference's
    own set-up at stencil orders 1 and 3 (tests/golden/fvm_orders_reference.npz)."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "fvm_orders_reference.npz")))
    q = lambda k: g["p%d_%s" % (p, k)]
    vr, vt, x, vmax = q("vr"), q("vt"), q("x"), float(q("domain")[1])
    for k, b in F.fvm_upwind_bands(vr, vt, x, p, p, p, vmax).items():
        assert np.max(np.abs(b - q(k))) <= 1e-12 * np.max(np.abs(q(k))), k
    Ep, En = F.adv_v_fvm(vr, vt, p, p, vmax)
    for mine, k in ((Ep, "op_adv_v_Ep"), (En, "op_adv_v_En")):
        assert np.max(np.abs(float(q("cA")) * mine - q(k))) <= 1e-12 * np.max(np.abs(q(k))), k
    xs = F.x_shift_bands(vr, vt, x, p, float(q("ax")), float(q("dt")))
    assert np.max(np.abs(xs - q("bte_x_shift_diag"))) <= 1e-12 * np.max(np.abs(q("bte_x_shift_diag")))
