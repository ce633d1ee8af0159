"""The GPU solve at the benchmarked shapes against golden EDFs from the reference itself.

Fixtures (tests/golden/make_golden_c2.py runs the reference's own bte_0d3v_batched, CPU path):
  * c2 shape: 128 B-splines x l_max 2 (n = 384), e-e on, 8 points; three at E/N < 10 Td with
    ionization degree above 1e-4, where the Coulomb term dominates;
  * reduced c5: 64 B-splines x l_max 4 (n = 320), e-e on, 4 points, ionization 1e-6..1e-2.
Each runs the reference driver's sequence (Maxwellian, e-e-off solve, e-e-on solve from it).

Tolerances:
  * plain FP64 form: 1e-10 relative L2 on the normalized EDF and relative on mean energy,
    mobility, diffusion and rates (rates with a floor of 1e-12 of the largest rate), on every
    point the reference converged (its final residual <= 1e-12 of its initial one);
  * a point where the reference stopped above that (its batch-global loop ended at its
    100-iteration cap): the GPU's FP64 solution must have a smaller residual in the
    reference's own metric, and the EDFs agree to the accuracy that residual allows,
    1e-10 x (reference rel_error / 1e-12);
  * mixed form: its EDF error against the reference is stated per point and bounded by 1e-8.
"""
import os

import numpy as np
import pytest

from helpers import gpu_solver, rel_l2_cols

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ATOL, RTOL = 1e-20, 1e-14


def _solve(s, args, g, P):
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, g[k])
    f0 = s.initialize(0, P)
    args.ee_collisions = 0
    f0, _ = s.solve(0, f0, ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)
    args.ee_collisions = 1
    return s.solve(0, f0, ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)


def _qoi_err(q, g):
    out = {k: np.abs(np.asarray(q[k]) - g[k]) / np.abs(g[k]) for k in ("energy", "mobility", "diffusion")}
    floor = 1e-12 * np.max(np.abs(g["rates"]), axis=0, keepdims=True)
    out["rates"] = np.max(np.abs(np.asarray(q["rates"]) - g["rates"]) / np.maximum(np.abs(g["rates"]), floor), axis=0)
    return out


def _tolerances(g, base):
    """Per-point EDF tolerance: `base` where the reference converged, scaled by its stated
    final residual where it stopped above 1e-12."""
    return base * np.maximum(1.0, g["rel_error"] / 1e-12)


@pytest.mark.parametrize("fixture,n_sp,l_max", [("c2_shape_reference.npz", 128, 2),
                                                ("c5_reduced_reference.npz", 64, 4)])
def test_fp64_against_reference(synthetic_xs, fixture, n_sp, l_max):
    g = dict(np.load(os.path.join(GOLDEN, fixture)))
    P = g["ff"].shape[1]
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, "fp64")
    ff, q = _solve(s, args, g, P)
    status = np.asarray(q["status"])
    err = rel_l2_cols(ff, g["ff"])
    qe = _qoi_err(q, g)
    print("\n%s fp64: EDF err %s\n  status %s, GPU rel_error %s, reference rel_error %s" % (
        fixture, np.array2string(err, precision=2), status, np.array2string(np.asarray(q["rel_error"]), precision=2),
        np.array2string(g["rel_error"], precision=2)))
    for k, v in qe.items():
        print("  %s err %s" % (k, np.array2string(v, precision=2)))
    assert np.all(status <= 1), status
    conv = g["rel_error"] <= 1e-12
    assert np.all(err[conv] < 1e-10), err
    for k, v in qe.items():
        assert np.all(v[conv] < 1e-10), (k, v)
    # where the reference stopped short, the GPU goes at least as far, and agrees to what
    # the reference's residual resolves
    short = ~conv
    assert np.all(np.asarray(q["rel_error"])[short] <= g["rel_error"][short]), q["rel_error"]
    assert np.all(err[short] < _tolerances(g, 1e-10)[short]), err


@pytest.mark.parametrize("fixture,n_sp,l_max", [("c2_shape_reference.npz", 128, 2),
                                                ("c5_reduced_reference.npz", 64, 4)])
def test_fp64_ee_off_against_reference(synthetic_xs, fixture, n_sp, l_max):
    """The first phase of the driver sequence alone (e-e off, from the Maxwellian) against the
    reference's e-e-off EDFs."""
    g = dict(np.load(os.path.join(GOLDEN, fixture)))
    P = g["ff"].shape[1]
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, "fp64")
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, g[k])
    args.ee_collisions = 0
    ff, q = s.solve(0, s.initialize(0, P), ATOL, RTOL, 100, "steady-state", 1e-16, 0.5, 1e-4)
    err = rel_l2_cols(ff, g["ff_warm"])
    print("\n%s fp64 e-e off: EDF err %s" % (fixture, np.array2string(err, precision=2)))
    assert np.all(np.asarray(q["status"]) <= 1)
    assert np.all(err < 1e-10), err


@pytest.mark.parametrize("fixture,n_sp,l_max", [("c2_shape_reference.npz", 128, 2),
                                                ("c5_reduced_reference.npz", 64, 4)])
def test_mixed_against_reference(synthetic_xs, fixture, n_sp, l_max):
    g = dict(np.load(os.path.join(GOLDEN, fixture)))
    P = g["ff"].shape[1]
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, "mixed")
    ff, q = _solve(s, args, g, P)
    status = np.asarray(q["status"])
    err = rel_l2_cols(ff, g["ff"])
    print("\n%s mixed: EDF err vs reference %s, status %s" % (fixture, np.array2string(err, precision=2), status))
    assert np.all(status <= 1), status
    assert np.all(err < np.maximum(1e-8, _tolerances(g, 1e-10))), err
    qe = _qoi_err(q, g)
    conv = g["rel_error"] <= 1e-12
    for k, v in qe.items():
        assert np.all(v[conv] < 1e-8), (k, v)
