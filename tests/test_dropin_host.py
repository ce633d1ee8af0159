"""Host-side methods of the drop-in class bte_0d3v_batched that need no GPU: the reference's
flop model (against values produced by the reference's own class, tests/golden/flops_reference.json)
and the scale of normalized_distribution (against the reference's converged c1 EDF)."""
import json
import os
import types

import numpy as np
import pytest

from boltzmann_gb300.bte_0d3v_batched import bte_0d3v_batched, normalization_scale
from boltzmann_gb300.workloads import EV_MAX, TE_NORM

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("ee", [0, 1])
def test_flop_model_matches_the_reference(synthetic_xs, ee):
    ref = json.load(open(os.path.join(HERE, "golden", "flops_reference.json")))["ee%d" % ee]
    args = types.SimpleNamespace(threads=1, sp_order=3, spline_qpts=5, ee_collisions=ee, verbose=0, use_gpu=1,
                                 Efreq=0.0, dt=1e-3, cycles=1, solver_type="steady-state", l_max=1, Nr=63, n_pts=1)
    s = bte_0d3v_batched(args, np.array([EV_MAX]), np.array([TE_NORM]), np.array([63]), [[[0, 0], [1, 0]]], 1,
                         [synthetic_xs])
    res, jac = s.rhs_and_jac_flops()
    for n, p, r, j in ref:
        assert (res(n, p), jac(n, p)) == (r, j), (n, p)


def test_normalization_scale_matches_the_reference():
    """The reference's converged c1 EDF is normalized: scaling it by 3.7 and normalizing again
    returns it, and its own scale is one."""
    g = dict(np.load(os.path.join(HERE, "golden", "c1_reference.npz")))
    from boltzmann_gb300.bte_1d3v_fvm import thermal_velocity
    vth = thermal_velocity(TE_NORM)
    ff = g["ff"]
    np.testing.assert_allclose(normalization_scale(g["mass_op"], ff, vth), 1.0, rtol=1e-12)
    f2 = 3.7 * ff
    np.testing.assert_allclose(f2 / normalization_scale(g["mass_op"], f2, vth), ff, rtol=1e-12, atol=0)


def test_spectral_1d3v_qoi_rows_and_arithmetic(synthetic_xs):
    """bte_1d3v.compute_qoi's rows and arithmetic on the host, with the oracle's operators of the
    1D3V golden grid (16 B-splines, l_max 1, plain knots) and its ordinate-to-harmonic
    projection, against the reference's compute_qoi (tests/golden/qoi_1d3v_reference.npz)."""
    from boltzmann_gb300.bte_1d3v import spectral_qoi_rows
    from boltzmann_gb300.bte_1d3v_fvm import qoi_from_moments
    from oracle import bte_oracle as O
    g = dict(np.load(os.path.join(HERE, "golden", "bte1d_reference.npz")))
    q = dict(np.load(os.path.join(HERE, "golden", "qoi_1d3v_reference.npz")))
    ops = O.Operators(O.processes_from_lxcat(synthetic_xs), 80.0, 4.0, 16, 1, ee=False, snap=False)
    np.testing.assert_allclose(ops.op_mass, g["op_mass"], rtol=0, atol=1e-14 * np.abs(g["op_mass"]).max())
    Q = spectral_qoi_rows(ops.op_mass, ops.op_temp, ops.op_rate, ops.vth, 2)
    Po = g["op_po2sh"]                                   # (nsh, Nvt)
    for k in ("v0", "v1", "v3"):
        V = g[k].reshape(16, Po.shape[1], -1)            # (Nr, Nvt, Nx)
        U = np.einsum("lj,rjx->rlx", Po, V).reshape(16 * 2, -1)
        out = qoi_from_moments(Q @ U, ops.vth, float(g["np0"]), np.sqrt(4 * np.pi))
        for name in ("rates", "ne", "Te"):
            ref = q["spec_%s_%s" % (k, name)]
            assert np.max(np.abs(out[name] - ref)) <= 1e-12 * np.max(np.abs(ref)), (k, name)


def test_checkpoint_round_trip(tmp_path):
    """write_checkpoint / read_checkpoint keep the reference's dataset names and values."""
    from boltzmann_gb300.bte_1d3v import read_checkpoint, write_checkpoint
    rng = np.random.default_rng(2)
    v, ne, Te = rng.random((20, 6)), rng.random(6), rng.random(6)
    pre = str(tmp_path / "cp_00001")
    write_checkpoint(pre, v, 0.25, 1e-3, ne, Te)
    t, dt, v2 = read_checkpoint(pre)
    assert (t, dt) == (0.25, 1e-3) and np.array_equal(v2, v)
    with np.load(pre + ".npz") as F:
        assert sorted(F.files) == sorted(["time[T]", "dt[T]", "edf", "ne[m^-3]", "Te[eV]"])
        assert np.array_equal(F["ne[m^-3]"], ne) and np.array_equal(F["Te[eV]"], Te)


def test_anisotropic_initial_state_matches_the_reference():
    """init_type "anisotropic" from the Maxwellian against the reference's own
    initialize(..., "anisotropic") (tests/golden/init_reference.npz), l_max 1 and 2."""
    from boltzmann_gb300.bte_0d3v_batched import anisotropic_from_maxwellian
    g = dict(np.load(os.path.join(HERE, "golden", "init_reference.npz")))
    for n_sp, l_max in ((64, 1), (16, 2)):
        ref = g["anisotropic_%d_%d" % (n_sp, l_max)]
        out = anisotropic_from_maxwellian(g["maxwellian_%d_%d" % (n_sp, l_max)], l_max + 1)
        assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref)), (n_sp, l_max)
