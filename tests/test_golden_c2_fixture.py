"""The benchmarked-shape fixtures' own records (no GPU): where the reference's answer is its
own exact fixed point and where it stops short (tests/golden/make_golden_c2.py --exact)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(fixture):
    return dict(np.load(os.path.join(GOLDEN, fixture)))


def _coulomb_dominated(g):
    return (g["EbyN"] < 10.0) & (g["ion_deg"] > 1e-4)


def test_reference_stops_short_where_coulomb_dominates():
    """The exact fixed point differs from the reference's answer only where the Coulomb term
    dominates (the reference's Newton omits two Jacobian terms and stops at its FP64 floor), by
    2e-6 at the c2 shape's first point; elsewhere, and in the e-e-off phase, the reference's
    answer is its fixed point to 1e-11."""
    g = _load("c2_shape_reference.npz")
    dom = _coulomb_dominated(g)
    assert g["exact_shift"][0] > 1e-6
    assert np.all(g["exact_shift"][~dom] < 1e-11)
    assert np.all(g["warm_exact_shift"] < 1e-11)


def test_device_potentials_shift_is_rounding_level():
    """The reference's answer with the device library's Rosenbluth potentials moves by at most a
    few 1e-10 (the determinacy of these points under rounding-level potential changes) and by
    the same amount as the exact fixed point of that system."""
    g = _load("c2_shape_reference.npz")
    assert np.all(g["rosenbluth_swap_shift"] < 2e-8)
    dom = _coulomb_dominated(g)
    assert np.all(g["rosenbluth_swap_shift"][~dom] < 5e-10)
    d = np.linalg.norm(g["ff_device_rosenbluth"] - g["ff_exact_device_rosenbluth"], axis=0) / np.linalg.norm(
        g["ff_exact_device_rosenbluth"], axis=0)
    assert np.all(d[~dom] < 1e-11), d
