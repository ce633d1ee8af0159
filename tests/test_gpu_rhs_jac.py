"""get_rhs_and_jacobian and the single transient step against the reference's own
(tests/golden/make_golden_rhs_jac.py: 16 B-splines, l_max 2, 3 points, e-e on and off).

The reference's closures are projected on its constraint basis Q, whose column signs depend on
the LAPACK build that computed the QR. The comparisons therefore use the sign-free n-space
forms Q y (residual) and Q J Q^T (Jacobian), and the step's new state v. Tolerance: 1e-8
relative to the largest entry; the library's M^-1 agrees with the reference's to about 1e-9
(the mass matrix's condition number times the rounding unit), and the M^-1-scaled operators
inherit that.
"""
import os

import numpy as np
import pytest

from helpers import gpu_solver

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(GOLDEN, "rhs_jac_reference.npz")))


def _solver(xs, g):
    s, args = gpu_solver(xs, 16, 2, True, 3, "fp64")
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, g[k])
    return s, args


@pytest.mark.parametrize("ee", [0, 1], ids=["ee_off", "ee_on"])
def test_rhs_and_jacobian_match_reference(synthetic_xs, golden, ee):
    g = golden
    s, args = _solver(synthetic_xs, g)
    args.ee_collisions = ee
    res, jac = s.get_rhs_and_jacobian(0, 3)
    Q = s._projected_ops(0)["Q"].cpu().numpy()
    Qr = g["qmat"]
    assert _rel(Q @ Q.T, Qr @ Qr.T) < 1e-12            # the same constrained subspace
    y = res(g["x"], 0.0, 0.0)
    J = jac(g["x"], 0.0, 0.0)
    tag = "ee" if ee else "noee"
    e_res = _rel(Q @ y, Qr @ g["res_" + tag])
    e_jac = _rel(np.einsum("ab,pbc,dc->pad", Q, J, Q), np.einsum("ab,pbc,dc->pad", Qr, g["jac_" + tag], Qr))
    print("\nrhs/jac (%s): residual %.2e, Jacobian %.2e" % (tag, e_res, e_jac))
    assert y.shape == g["res_" + tag].shape and J.shape == g["jac_" + tag].shape
    assert e_res < 1e-8 and e_jac < 1e-8


def test_step_matches_reference(synthetic_xs, golden):
    g = golden
    s, args = _solver(synthetic_xs, g)
    args.ee_collisions, args.Efreq = 1, 13.56e6
    v = s.step(0, g["x"], 1e-30, 1e-12, 50, 0.0, float(g["step_dt"]))
    err = _rel(v, g["step_v"])
    print("\nstep: %.2e (state change %.2e)" % (err, _rel(g["step_v"], g["x"])))
    assert err < 1e-8


def test_rhs_jacobian_tensor_in_tensor_out(synthetic_xs, golden):
    import torch
    g = golden
    s, args = _solver(synthetic_xs, g)
    args.ee_collisions = 1
    res, jac = s.get_rhs_and_jacobian(0, 3)
    x = torch.as_tensor(g["x"], device="cuda")
    y, J = res(x, 0.0, 0.0), jac(x, 0.0, 0.0)
    assert torch.is_tensor(y) and y.is_cuda and torch.is_tensor(J) and J.is_cuda
    assert np.array_equal(y.cpu().numpy(), res(g["x"], 0.0, 0.0))
