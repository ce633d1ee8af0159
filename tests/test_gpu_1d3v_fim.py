"""Fully implicit spectral 1D3V step on the GPU against the oracle.

The reference has no fully implicit solver for the spectral v-space (its fully implicit step
asserts the finite-volume one, BESolver/python/bte_1d3v_solver.py:1891). The oracle composes
the coupled operator from the reference's operators as the reference's matvec test composes it
(test_bte_1d_matvec.py:19-83) and solves the step directly; its operators are pinned to the
reference's own 1D3V fixture (tests/test_gpu_1d3v.py, tests/test_oracle_golden.py). The grid
is that fixture's: 16 Chebyshev points, 16 B-splines, l_max 1, 8 ordinates (2048 unknowns).
Tolerances: matvec 1e-12 relative to the largest entry; the GMRES step (rtol 1e-12) 1e-9."""
import ast
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "bte1d_reference.npz")


def rel(a, b):
    a = a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def case(synthetic_xs):
    from boltzmann_gb300.bte_1d3v import bte_1d3v
    from oracle.bte1d_oracle import Oracle1D
    g = {k: np.real(v) if np.iscomplexobj(v) else v for k, v in np.load(GOLD).items()}
    p = ast.literal_eval(str(g["params"]))
    p = dict(p, collisions=synthetic_xs, solver_type="fully_implicit")
    b = bte_1d3v(p)
    o = Oracle1D(synthetic_xs, p["Np"], p["Nr"], p["Nvt"], p["lmax"], p["ev_max"], p["Te"], p["L"], p["freq"],
                 p["Tg"], p["p0"])
    return b, o, g, p


def test_fim_matvec_against_oracle(case):
    b, o, g, p = case
    rng = np.random.default_rng(3)
    v = rng.standard_normal((b.dof_vr * b.dof_vt, b.dof_x))
    for E in (g["E"], np.zeros(b.dof_x)):
        y = b.fim_mvec(E, v, p["dt"])
        assert rel(y, v - p["dt"] * o.rhs_vx(E, v)) < 1e-12


@pytest.mark.parametrize("pc", ["split", "vblock"])
def test_fim_step_against_direct_solve(case, pc):
    """GMRES to rtol 1e-12 reaches the oracle's direct solve; more than one Krylov iteration is
    needed, since neither preconditioner is the exact inverse of the coupled operator."""
    b, o, g, p = case
    v0 = g["v0"]
    for dt in (p["dt"], 10 * p["dt"]):
        v1 = b.step_fim(g["E"], v0, 0.0, dt, rtol=1e-12, atol=1e-30, pc=pc)
        ref = o.step_fim(g["E"], v0, dt)
        assert rel(v1, ref) < 1e-9, (pc, dt, rel(v1, ref))
        info = b.gmres_info
        assert info["status"] == 0 and info["iterations"] > 1 and info["residual_rel"] <= 1e-12
        print("\npc %s dt %g: %d GMRES iterations" % (pc, dt, info["iterations"]))


def test_fim_step_keeps_inflow_zero(case):
    b, o, g, p = case
    v1 = b.step(g["E"], g["v0"], None, 0.0, p["dt"]).cpu().numpy().reshape(b.dof_vr, b.dof_vt, b.dof_x)
    left, right = o.inflow_rows()
    assert np.all(v1[:, left, 0] == 0.0) and np.all(v1[:, right, -1] == 0.0)
