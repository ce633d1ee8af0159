"""The GPU solve at the benchmarked shapes against golden EDFs from the reference itself.

Fixtures (tests/golden/make_golden_c2.py runs the reference's own bte_0d3v_batched, CPU path):
  * c2 shape: 128 B-splines x l_max 2 (n = 384), e-e on, 8 points; the first three at E/N < 10
    Td with ionization degree above 1e-4, where the Coulomb term dominates;
  * reduced c5: 64 B-splines x l_max 4 (n = 320), e-e on, 4 points, ionization 1e-6..1e-2; the
    first (1.2 Td, 8e-3) Coulomb-dominated.
Each runs the reference driver's sequence (Maxwellian, e-e-off solve, e-e-on solve from it).

Besides the reference's answers the fixtures hold what bounds agreement with them:
  * `ff_warm_exact`, `ff_exact`: the exact fixed points of the reference's own discrete
    systems (its residual in extended precision, full Newton). The reference's Newton leaves
    two rank-one terms out of its Jacobian and stops at its FP64 floor; at the c2 shape's first
    point its answer is 2.0e-6 from its own fixed point (`exact_shift`).
  * `ff_device_rosenbluth` (c2): the reference's answer with its Rosenbluth potentials
    replaced by the device library's, which agree with its own to 2e-14 of their largest
    entry; `rosenbluth_swap_shift` is how far that moves the reference (up to 2.2e-10 here),
    the FP64 determinacy of these points under rounding-level changes of the potentials;
    `ff_exact_device_rosenbluth` is the exact fixed point of that system.

Tolerances (relative L2 of the normalized EDF; QoIs relative):
  * e-e off, plain FP64: 1e-10 against the exact e-e-off fixed point, every point;
  * e-e on, plain FP64, points not Coulomb-dominated: 1e-10 against the reference's answer
    built on the same potentials where the fixture has it (c2), else against the reference's
    own answer; mean energy, mobility and diffusion to 1e-10 plus the potentials' shift;
  * e-e on, Coulomb-dominated points: against the exact fixed point of the system on the
    device potentials, the plain FP64 form's own resolution at that workload: 1e-7 at the c2
    shape (over the 4096-point c2 batch its answers from two starting points differ by up to
    9.3e-8) and 1e-6 at the reduced c5 shape (over 2048 c5 points, a median of 1.25e-6 at the
    points where the two forms differ by more than 1e-6). Measured: 1.6e-8 (c2) and 1.9e-7
    (c5) from the exact fixed point, where the reference's own answer is 2.0e-6 and 1.9e-9 away;
  * mixed form: the same bounds, each point's error stated.
"""
import os

import numpy as np
import pytest

from helpers import gpu_solver, rel_l2_cols

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ATOL, RTOL = 1e-20, 1e-14
FIXTURES = [("c2_shape_reference.npz", 128, 2), ("c5_reduced_reference.npz", 64, 4)]
# bound at the Coulomb-dominated points: the plain FP64 form's own resolution there
DOMINATED_TOL = {"c2_shape_reference.npz": 1e-7, "c5_reduced_reference.npz": 1e-6}


def _load(fixture):
    return dict(np.load(os.path.join(GOLDEN, fixture)))


def _solve(s, args, g, P):
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, g[k])
    f0 = s.initialize(0, P)
    args.ee_collisions = 0
    ffw, _ = s.solve(0, f0, ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)
    args.ee_collisions = 1
    ff, q = s.solve(0, ffw, ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)
    return np.asarray(ffw), np.asarray(ff), q


def _coulomb_dominated(g):
    return (g["EbyN"] < 10.0) & (g["ion_deg"] > 1e-4)


def _check_ee_on(g, ff, q, label, dom_tol):
    """EDF and QoI bounds of the e-e-on solve (module docstring)."""
    dom = _coulomb_dominated(g)
    target = g.get("ff_device_rosenbluth", g["ff"])
    shift = g.get("rosenbluth_swap_shift", np.zeros(len(dom)))
    err_ref = rel_l2_cols(ff, g["ff"])
    err_same = rel_l2_cols(ff, target)
    exact = g.get("ff_exact_device_rosenbluth", g["ff_exact"])
    err_exact = rel_l2_cols(ff, exact)
    print("\n%s: EDF err vs reference %s\n  vs reference on the device potentials %s\n  vs exact fixed point %s\n"
          "  reference vs exact %s, Coulomb-dominated %s" % (
              label, np.array2string(err_ref, precision=2), np.array2string(err_same, precision=2),
              np.array2string(err_exact, precision=2), np.array2string(g["exact_shift"], precision=2), dom))
    assert np.all(np.asarray(q["status"]) <= 1), q["status"]
    assert np.all(err_same[~dom] < 1e-10), err_same
    assert np.all(err_ref[~dom] < 1e-10 + shift[~dom]), err_ref
    assert np.all(err_exact[dom] < dom_tol), err_exact
    for k in ("energy", "mobility", "diffusion"):
        e = np.abs(np.asarray(q[k]) - g[k]) / np.abs(g[k])
        assert np.all(e[~dom] < 1e-10 + 2.0 * shift[~dom]), (k, e)


@pytest.mark.parametrize("fixture,n_sp,l_max", FIXTURES)
def test_fp64_ee_off_against_exact(synthetic_xs, fixture, n_sp, l_max):
    """The first phase of the driver sequence (e-e off, from the Maxwellian) against the exact
    e-e-off fixed point and the reference's answer (within 1e-10 plus its own distance from it)."""
    g = _load(fixture)
    P = g["ff"].shape[1]
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, "fp64")
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, g[k])
    args.ee_collisions = 0
    ff, q = s.solve(0, s.initialize(0, P), ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)
    ff = np.asarray(ff)
    err_exact = rel_l2_cols(ff, g["ff_warm_exact"])
    err_ref = rel_l2_cols(ff, g["ff_warm"])
    print("\n%s fp64 e-e off: EDF err vs exact %s, vs reference %s" % (
        fixture, np.array2string(err_exact, precision=2), np.array2string(err_ref, precision=2)))
    assert np.all(np.asarray(q["status"]) <= 1)
    assert np.all(err_exact < 1e-10), err_exact
    assert np.all(err_ref < 1e-10 + g["warm_exact_shift"]), err_ref


@pytest.mark.parametrize("fixture,n_sp,l_max", FIXTURES)
def test_fp64_against_reference(synthetic_xs, fixture, n_sp, l_max):
    g = _load(fixture)
    P = g["ff"].shape[1]
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, "fp64")
    _, ff, q = _solve(s, args, g, P)
    _check_ee_on(g, ff, q, fixture + " fp64", DOMINATED_TOL[fixture])


@pytest.mark.parametrize("fixture,n_sp,l_max", FIXTURES)
def test_mixed_against_reference(synthetic_xs, fixture, n_sp, l_max):
    g = _load(fixture)
    P = g["ff"].shape[1]
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, "mixed")
    _, ff, q = _solve(s, args, g, P)
    _check_ee_on(g, ff, q, fixture + " mixed", DOMINATED_TOL[fixture])

