"""The finite-volume 1D3V set-up on the host (grids, upwind operators and bands, the factored
collision operator and its closed-form inverse) against the reference's own set-up
(tests/golden/fvm_reference.npz) and the oracle."""
import os

import numpy as np
import pytest

from boltzmann_gb300 import bte_1d3v_fvm as P
from boltzmann_gb300.bte_1d3v import ordinates
from boltzmann_gb300.lxcat import read_cross_section_data
from oracle import bte1d_fvm_oracle as F

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fvm_reference.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


def test_grids_match_the_reference(g):
    vr, qw, vmax = P.radial_cells(80.0, 4.0, 7, 3, int(g["spline_qpts"]))
    np.testing.assert_allclose(vr, g["vr"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(qw, g["vr_qw"], rtol=1e-15, atol=0)
    assert vmax == pytest.approx(float(g["domain"][1]), rel=1e-15)
    vt, vt_qw = ordinates(int(g["Nvt"]))
    np.testing.assert_allclose(vt, g["vt"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(vt_qw, g["vt_qw"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(P.x_points(int(g["Nx"])), g["x"], rtol=0, atol=1e-15)
    assert np.array_equal(P.x_points(5, adaptive_grid=0), np.linspace(-1, 1, 5))


def test_fd_weights_are_exact_on_polynomials():
    rng = np.random.default_rng(3)
    for n in (2, 3, 4, 5):
        nodes = np.sort(rng.uniform(-1.0, 2.0, n))
        x0 = nodes[rng.integers(n)]
        w = P.fd_weights(x0, nodes)
        for p in range(n):
            exact = p * x0 ** (p - 1) if p else 0.0
            assert abs(w @ nodes ** p - exact) <= 1e-9 * max(1.0, abs(exact))


def test_upwind_operators_match_the_reference_and_the_oracle(g):
    """Fornberg weights against the reference's operators (inflow rows zeroed, as captured) and
    the oracle's explicit Lagrange-derivative weights."""
    for D, x, sw, dirn, theta in ((g["Dx_LtoR"], g["x"], int(g["px"]) + 1, "L", False),
                                  (g["Dx_RtoL"], g["x"], int(g["px"]) + 1, "R", False),
                                  (g["Dvt_LtoR"], g["vt"], int(g["pvt"]) + 1, "L", True),
                                  (g["Dvt_RtoL"], g["vt"], int(g["pvt"]) + 1, "R", True)):
        mine = (P.upwind_operator_theta if theta else P.upwind_operator)(x, sw, dirn)
        orc = (F.upwind_d1_theta if theta else F.upwind_d1)(np.asarray(x), sw, dirn)
        assert np.max(np.abs(mine - orc)) <= 1e-12 * np.max(np.abs(orc))
        mine[0 if dirn == "L" else -1, :] = 0.0
        assert np.max(np.abs(mine - D)) <= 1e-12 * np.max(np.abs(D))


def test_bands_match_the_reference(g):
    p = [int(g[k]) for k in ("pvr", "pvt", "px")]
    ops = P.fvm_upwind_operators(g["vr"], g["vt"], g["x"], *p, float(g["domain"][1]))
    for k, b in P.fvm_bands(ops, *p).items():
        assert b.shape == g[k].shape
        assert np.max(np.abs(b - g[k])) <= 1e-13 * np.max(np.abs(g[k])), k


def test_collision_operator_and_closed_form_inverse(g, synthetic_xs):
    """The factored operator reproduces the reference's op_col_en; its closed-form inverse the
    reference's dense PmatC; `apply` the dense product."""
    procs = list(read_cross_section_data(synthetic_xs).values())
    vt, vt_qw = ordinates(int(g["Nvt"]))
    gain, loss = P.fvm_collisions(procs, g["vr"], vt_qw, float(g["vth"]), float(g["domain"][1]))
    C = P.FvmCollisions(gain, loss, 2.0 * np.pi * vt_qw)
    ref = g["op_col_en"]
    assert np.max(np.abs(C.dense() - ref)) <= 1e-13 * np.max(np.abs(ref))
    c = float(g["dt"]) * float(g["tau"]) * float(g["n0"]) * float(g["np0"])
    Pm = C.inverse_dense(c)
    assert np.max(np.abs(Pm - g["PmatC"])) <= 1e-12 * np.max(np.abs(g["PmatC"]))
    v = np.random.default_rng(1).standard_normal((C.Nr * C.Nvt, 3))
    np.testing.assert_allclose(C.apply(v), C.dense() @ v, rtol=0, atol=1e-13 * np.abs(C.dense() @ v).max())
    # (I - c C) applied to the inverse's output returns the input
    y = Pm @ v
    np.testing.assert_allclose(y - c * C.apply(y), v, rtol=0, atol=1e-12 * np.abs(v).max())


def test_attachment_has_no_fvm_operator(g):
    proc = {"type": "ATTACHMENT", "threshold": 0.0, "energy": [0.0, 1.0], "cross section": [1e-20, 1e-20]}
    with pytest.raises(NotImplementedError):
        P.fvm_collisions([proc], g["vr"], np.ones(4), float(g["vth"]), float(g["domain"][1]))


def test_setup_from_the_parameter_table(synthetic_xs, g):
    """fvm_setup on the fixtures' parameter table reproduces the reference's grids, bands and
    collision operator."""
    from helpers import FVM_IMPLICIT_PARAMS
    st = P.fvm_setup(dict(FVM_IMPLICIT_PARAMS, collisions=synthetic_xs))
    for k in ("vr", "vt", "x"):
        np.testing.assert_allclose(st.grid_info[k], g[k], rtol=0, atol=1e-14 * np.abs(g[k]).max())
    for k, b in st.bands.items():
        assert np.max(np.abs(b - g[k])) <= 1e-13 * np.max(np.abs(g[k])), k
    assert np.max(np.abs(st.collisions.dense() - g["op_col_en"])) <= 1e-13 * np.max(np.abs(g["op_col_en"]))
    p = st.params
    assert p.L == pytest.approx(float(g["L"])) and p.tau == pytest.approx(float(g["tau"]))
    assert p.n0 == pytest.approx(float(g["n0"]), rel=1e-14) and p.solver == "fully_implicit"


@pytest.mark.parametrize("change", [dict(vspace_type=1), dict(pc_type="xvx_solve"), dict(solver_type="xvx_strang_split"),
                                    dict(ic_file="ic.h5"), dict(xspace_type=2), dict(xspace_type=1)])
def test_setup_refuses_what_is_not_provided(synthetic_xs, change):
    from helpers import FVM_IMPLICIT_PARAMS
    with pytest.raises((NotImplementedError, ValueError)):
        P.fvm_setup(dict(FVM_IMPLICIT_PARAMS, collisions=synthetic_xs, **change))


def test_initial_condition_matches_the_reference(synthetic_xs):
    from helpers import FVM_IMPLICIT_PARAMS
    gi = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "fvm_implicit_reference.npz")))
    st = P.fvm_setup(dict(FVM_IMPLICIT_PARAMS, collisions=synthetic_xs))
    v = P.fvm_initial_condition(st.params, st.vth, st.vr, len(st.vt), st.x)
    assert np.max(np.abs(v - gi["v0"])) <= 1e-14 * np.max(np.abs(gi["v0"]))


def test_qoi_functionals_and_compute_qoi_match_the_reference(synthetic_xs):
    """The FVM QoI rows and compute_qoi's arithmetic (on the host, from Q v) against the
    reference's op_mass/op_temp/op_rate and compute_qoi (tests/golden/qoi_1d3v_reference.npz)."""
    from helpers import FVM_IMPLICIT_PARAMS
    q = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi_1d3v_reference.npz")))
    st = P.fvm_setup(dict(FVM_IMPLICIT_PARAMS, collisions=synthetic_xs))
    for i, ref in enumerate([q["fvm_op_mass"], q["fvm_op_temp"]] + list(q["fvm_op_rate"])):
        assert np.max(np.abs(st.qoi[i] - ref)) <= 1e-14 * np.max(np.abs(ref)), i
    for k in ("v0", "vp"):
        out = P.qoi_from_moments(st.qoi @ q["fvm_%s" % k], st.vth, st.params.np0, 1.0)
        for name in ("rates", "ne", "Te"):
            ref = q["fvm_%s_%s" % (k, name)]
            assert np.max(np.abs(out[name] - ref)) <= 1e-13 * np.max(np.abs(ref)), (k, name)


def test_radial_components_match_the_reference(synthetic_xs):
    """ords_to_sph's projection and compute_radial_components's interpolation on the FVM grid
    against the reference's (tests/golden/qoi_1d3v_reference.npz); speeds outside the cells
    raise as the reference's interpolation does."""
    from helpers import FVM_IMPLICIT_PARAMS
    from boltzmann_gb300.bte_1d3v import sph_ords_projections
    q = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi_1d3v_reference.npz")))
    st = P.fvm_setup(dict(FVM_IMPLICIT_PARAMS, collisions=synthetic_xs))
    _, po2sh = sph_ords_projections(st.vt, st.vt_qw, st.params.l_max)
    U = np.einsum("li,rix->rlx", po2sh, q["fvm_vp"].reshape(len(st.vr), len(st.vt), -1)).reshape(-1, len(st.x))
    assert np.max(np.abs(U - q["fvm_vp_sph"])) <= 1e-14 * np.max(np.abs(q["fvm_vp_sph"]))
    R = P.fvm_radial_components(U, st.vr, 2, q["ev"], st.vth)
    assert np.max(np.abs(R - q["fvm_vp_radial"])) <= 1e-14 * np.max(np.abs(q["fvm_vp_radial"]))
    with pytest.raises(ValueError):
        P.fvm_radial_components(U, st.vr, 2, np.array([79.9]), st.vth)


@pytest.mark.parametrize("p", [1, 3])
def test_bands_at_other_orders_match_the_reference(p):
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "fvm_orders_reference.npz")))
    q = lambda k: g["p%d_%s" % (p, k)]
    ops = P.fvm_upwind_operators(q("vr"), q("vt"), q("x"), p, p, p, float(q("domain")[1]))
    for k, b in P.fvm_bands(ops, p, p, p).items():
        assert b.shape == q(k).shape
        assert np.max(np.abs(b - q(k))) <= 1e-12 * np.max(np.abs(q(k))), k
