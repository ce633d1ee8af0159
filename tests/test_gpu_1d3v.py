"""1D3V spectral step on the GPU (boltzmann_gb300.bte_1d3v through include/bte1d_gb300.h)
against golden vectors of the reference's own step and against the oracle."""
import ast
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "bte1d_reference.npz")


def rel(a, b):
    a = a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
    b = np.real(b)  # the reference's eigenbasis is complex-typed with zero imaginary parts
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def case(synthetic_xs):
    from boltzmann_gb300.bte_1d3v import bte_1d3v
    g = {k: np.real(v) if np.iscomplexobj(v) else v for k, v in np.load(GOLD).items()}
    p = ast.literal_eval(str(g["params"]))
    b = bte_1d3v(dict(p, collisions=synthetic_xs))
    return b, g, p


@pytest.mark.parametrize("name", ["Dp", "xp_vt", "op_po2sh", "op_psh2o", "op_adv_x", "op_col_en", "op_col_gT",
                                  "op_adv_v"])
def test_setup_operators(case, name):
    b, g, _ = case
    assert rel(getattr(b, name), g[name]) < 1e-12


def test_initial_condition(case):
    b, g, _ = case
    assert rel(b.initial_condition(), g["v0"]) < 1e-12


def test_x_step(case):
    b, g, p = case
    assert rel(b.step_bte_x(g["v0"], 0.0, 0.5 * p["dt"]), g["v1"]) < 1e-11
    assert rel(b.step_bte_x(g["v2"], 0.0, 0.5 * p["dt"]), g["v3"]) < 1e-11


def test_v_step_gmres(case):
    """GMRES with the per-point FP32 block preconditioner reaches the reference's v-step within
    the two solvers' tolerances (rtol 1e-12 each) in a handful of iterations."""
    b, g, p = case
    v2 = b.step_bte_v(g["E"], g["v1"], None, 0.0, p["dt"])
    assert rel(v2, g["v2"]) < 1e-10
    assert b.gmres_info["status"] == 0 and b.gmres_info["iterations"] <= 8
    assert b.gmres_info["residual_rel"] < 1e-12


def test_strang_step(case):
    b, g, p = case
    assert rel(b.step(g["E"], g["v0"], None, 0.0, p["dt"]), g["v3"]) < 1e-10


def test_lmat_and_projections_against_oracle(case, synthetic_xs):
    from oracle.bte1d_oracle import Oracle1D
    b, g, p = case
    o = Oracle1D(synthetic_xs, p["Np"], p["Nr"], p["Nvt"], p["lmax"], p["ev_max"], p["Te"], p["L"], p["freq"],
                 p["Tg"], p["p0"])
    rng = np.random.default_rng(5)
    u = rng.standard_normal((b.dof_v, b.dof_x))
    assert rel(b.lmat_mvec(g["E"], u, p["dt"]), o.lmat(g["E"], u, p["dt"])) < 1e-13
    v = rng.standard_normal((b.dof_vr * b.dof_vt, b.dof_x))
    assert rel(b.ords_to_sph(v), o.ords_to_sph(v)) < 1e-13
    assert rel(b.sph_to_ords(u), o.sph_to_ords(u)) < 1e-13


def test_block_preconditioner(case, synthetic_xs):
    """The per-point FP32 block solve against NumPy, including the E = 0 and dt = 0 blocks
    (whose -0.0 entries once misled the FP32 pivot search)."""
    b, g, p = case
    n, Nx = b.dof_v, b.dof_x
    rng = np.random.default_rng(9)
    u = rng.standard_normal((n, Nx))
    Cv = p["dt"] * b._keep[7]
    Av = p["dt"] * b._keep[8]
    for E, dt in ((g["E"], p["dt"]), (np.zeros(Nx), p["dt"]), (np.zeros(Nx), 0.0)):
        y = b.block_solve(E, u, dt).cpu().numpy()
        f = dt / p["dt"]
        ref = np.stack([np.linalg.solve(np.eye(n) - f * (Cv + E[x] * Av), u[:, x]) for x in range(Nx)], axis=1)
        assert float(np.max(np.abs(y - ref)) / np.max(np.abs(ref))) < 1e-5
