"""GPU path directly against the golden vectors produced by the reference itself."""
import os

import numpy as np
import pytest

from helpers import gpu_solver, relmax

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ATOL, RTOL = 1e-20, 1e-14


def solve(s, args, g, ee, P):
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, g[k])
    f0 = s.initialize(0, P)
    if ee:
        args.ee_collisions = 0
        f0, _ = s.solve(0, f0, ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)
        args.ee_collisions = 1
    return s.solve(0, f0, ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_c1_against_reference(synthetic_xs, precision, tol):
    g = dict(np.load(os.path.join(GOLDEN, "c1_reference.npz")))
    s, args = gpu_solver(synthetic_xs, 64, 1, False, 1, precision)
    assert np.array_equal(s.export_operator(0, "KNOTS").cpu().numpy(), g["knots"])
    assert relmax(s.export_operator(0, "MASS").cpu().numpy(), g["mass_mat"]) < 1e-13
    assert relmax(s.initialize(0, 1), g["f0"]) < 1e-10
    ff, q = solve(s, args, g, False, 1)
    assert np.linalg.norm(ff - g["ff"]) / np.linalg.norm(g["ff"]) < tol
    for k in ("energy", "mobility", "diffusion"):
        assert relmax(q[k], g[k]) < tol
    floor = 1e-12 * np.max(np.abs(g["rates"]))
    assert np.max(np.abs(q["rates"] - g["rates"]) / np.maximum(np.abs(g["rates"]), floor)) < tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_ee_against_reference(synthetic_xs, precision, tol):
    g = dict(np.load(os.path.join(GOLDEN, "ee_small_reference.npz")))
    s, args = gpu_solver(synthetic_xs, 16, 2, True, 3, precision)
    n = s._grid_info[0]["n"]
    cca = np.zeros((n, n, n))
    cca[tuple(g["cc_a_idx"])] = g["cc_a_val"]
    assert relmax(s.export_operator(0, "CC_A").cpu().numpy(), cca) < 1e-12
    ff, q = solve(s, args, g, True, 3)
    err = np.linalg.norm(ff - g["ff"], axis=0) / np.linalg.norm(g["ff"], axis=0)
    assert np.max(err) < tol, err
    for k in ("energy", "mobility", "diffusion"):
        assert relmax(q[k], g[k]) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_transient_matches_reference(synthetic_xs, precision):
    """solve(..., "transient") on the GPU against the reference's own transient solve over one
    RF period (golden vectors); both stop each step's chord iteration at rtol 1e-10."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "transient_reference.npz"))
    s, args = gpu_solver(synthetic_xs, 32, 1, False, 2, precision=precision)
    args.dt, args.cycles, args.Efreq = float(g["dt"]), float(g["cycles"]), float(g["Efreq"])
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E", "eRe", "eIm"]:
        s.set_boltzmann_parameter(0, k, g[k])
    u, qoi = s.solve(0, g["f0"], 1e-30, 1e-10, 200, "transient")
    assert np.all(qoi["status"] == 0)
    assert relmax(u, g["u"]) < 1e-8
    for k in ("energy", "mobility", "diffusion"):
        assert np.max(np.abs(qoi[k] - g[k]) / np.abs(g[k])) < 1e-8
