"""Device-assembled operators against the CPU oracle (FP64, same inputs)."""
import numpy as np
import pytest

from helpers import gpu_solver, oracle_ops, relmax

pytestmark = pytest.mark.gpu

CASES = [(64, 1, False, 0), (24, 2, True, 0), (16, 4, True, 1)]


@pytest.fixture(scope="module", params=CASES, ids=lambda c: "nsp%d_l%d_ee%d_ext%d" % c)
def pair(request, synthetic_xs):
    n_sp, l_max, ee, ext = request.param
    s, _ = gpu_solver(synthetic_xs, n_sp, l_max, ee, 1, ext=ext)
    o = oracle_ops(synthetic_xs, n_sp, l_max, ee, ext=bool(ext))
    return s, o, ee


def exp(s, name):
    return s.export_operator(0, name).cpu().numpy()


def test_knots(pair):
    s, o, _ = pair
    assert np.array_equal(exp(s, "KNOTS"), o.knots)


@pytest.mark.parametrize("name,attr,tol", [
    ("MASS", "Mmat", 1e-13), ("ADV_RAW", "adv_raw", 1e-13),
    ("COL_GT_RAW", "FOp_g", 1e-12), ("MASS_VEC", "op_mass", 1e-13), ("TEMP_VEC", "op_temp", 1e-13),
    ("MOBILITY", "op_mobility", 1e-13), ("DIFFUSION", "op_diffusion", 1e-13), ("RATES", "op_rate", 1e-12)])
def test_operator(pair, name, attr, tol):
    s, o, _ = pair
    assert relmax(exp(s, name), getattr(o, attr)) < tol


def test_collision_operator(pair):
    s, o, _ = pair
    got = exp(s, "COL_RAW")
    for sp in range(len(o.FOp)):
        assert relmax(got[sp], o.FOp[sp]) < 1e-12


def test_inverse_mass_within_its_conditioning(pair):
    """M^-1 (Cholesky, then the inverse factor's product) against the oracle's, within what FP64
    determines of an inverse: a few eps times cond(M) relative to its largest entry. (On the
    c2-shape grid, 128 splines x l_max 2 with cond(M) = 5.7e6, the device's M^-1 and Rosenbluth
    potentials agree with the reference's own to 8e-16 and 2.4e-15 in the Frobenius norm.)"""
    s, o, _ = pair
    cond = float(np.linalg.cond(o.Mmat))
    err = relmax(exp(s, "MINV"), o.Minv)
    print("\nMINV relmax %.2e, cond(M) %.2e, bound %.2e" % (err, cond, 16 * np.finfo(float).eps * cond))
    assert err < max(1e-13, 16 * np.finfo(float).eps * cond)


def test_coulomb_operators(pair):
    s, o, ee = pair
    if not ee:
        pytest.skip("e-e off")
    cond = float(np.linalg.cond(o.Mmat))
    bound = max(1e-13, 16 * np.finfo(float).eps * cond)  # HL, GL carry M^-1
    eh, eg = relmax(exp(s, "HL"), o.hl_op), relmax(exp(s, "GL"), o.gl_op)
    print("\nHL relmax %.2e, GL relmax %.2e, bound %.2e" % (eh, eg, bound))
    assert eh < bound and eg < bound
    assert relmax(exp(s, "CC_A"), o.cc_a) < 1e-12
    assert relmax(exp(s, "CC_B"), o.cc_b) < 1e-12


def test_initial_state(pair):
    from oracle import bte_oracle as O
    s, o, _ = pair
    f0 = s.initialize(0, 3)
    ref = O.maxwellian_initial(o, 3)
    assert relmax(f0, ref) < 1e-10
