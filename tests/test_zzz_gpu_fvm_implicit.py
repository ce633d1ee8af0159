"""The finite-volume 1D3V fully implicit step on the GPU (boltzmann_gb300.bte_1d3v_fvm, the
library's bte_fvm_* entry points) against the reference's own operator, preconditioner and
step (tests/golden/fvm_implicit_reference.npz), with the product's own host set-up built from
the same parameter table. The file is named so that pytest collects it last, after the
parity tests of the batched solver."""
import os

import numpy as np
import pytest

from helpers import FVM_IMPLICIT_PARAMS as PARAMS

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fvm_implicit_reference.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="module")
def solver(synthetic_xs, g):
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    s = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs))
    assert (s.dof_vr, s.dof_vt, s.dof_x) == (int(g["Nr"]), int(g["Nvt"]), int(g["Nx"]))
    s.init(float(g["dt"]))
    return s


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b)) / np.max(np.abs(b)))


def test_grid_and_initial_condition(solver, g):
    for k in ("vr", "vt", "x"):
        np.testing.assert_allclose(solver.grid_info[k], g[k], rtol=0, atol=1e-14 * np.abs(g[k]).max())
    assert _rel(solver.initial_condition(0).cpu().numpy(), g["v0"]) <= 1e-13


def test_operator_matches_the_reference(solver, g):
    Y = solver.rhs_mvec(g["E"], g["u"].reshape(-1, int(g["Nx"])), float(g["dt"])).cpu().numpy().reshape(-1)
    assert _rel(Y, g["Au"]) <= 1e-12


def test_preconditioner_matches_the_reference_op_split_step(solver, g):
    Y = solver.step_op_split(g["E"], g["u"].reshape(-1, int(g["Nx"])), None, 0.0, float(g["dt"])).cpu().numpy()
    assert _rel(Y.reshape(-1), g["Mu"]) <= 1e-12


@pytest.mark.parametrize("pc_left", [False, True])
def test_step_matches_the_reference(solver, g, pc_left):
    n0 = solver.launches()
    y = solver.step(g["E"], g["v0"], None, 0.0, float(g["dt"]), pc_left=pc_left).cpu().numpy()
    assert solver.gmres_info["status"] == 0
    assert 0 < solver.gmres_info["iterations"] <= 100
    assert _rel(y, g["step"]) <= 1e-10
    assert solver.launches() > n0


def test_step_before_init_is_refused(synthetic_xs):
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    s = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs))
    with pytest.raises(RuntimeError):
        s.step(np.ones(s.dof_x), np.ones((s.dof_v, s.dof_x)), None, 0.0, 1e-3)


def test_semi_lagrangian_step_matches_the_reference(synthetic_xs):
    """solver_type "sl_implicit": the advection (step_adv_vx_sl) and the step against the
    reference's (tests/golden/fvm_sl_reference.npz)."""
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    from helpers import FVM_SL_PARAMS
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "fvm_sl_reference.npz")))
    s = bte_1d3v_fvm(dict(FVM_SL_PARAMS, collisions=synthetic_xs))
    dt = float(g["dt"])
    s.init(dt)
    v_sl = s.step_adv_vx_sl(g["E"], g["v0"], 0.0, dt).cpu().numpy()
    assert _rel(v_sl, g["v_sl"]) <= 1e-13
    y = s.step(g["E"], g["v0"], None, 0.0, dt).cpu().numpy()
    assert _rel(y, g["step"]) <= 1e-12


# ---- drop-in utilities of bte_0d3v_batched added with this file's path


def test_normalized_distribution_and_batched_inv(synthetic_xs):
    """normalized_distribution against the reference's converged (normalized) c1 EDF, and
    batched_inv against NumPy's inverse; a singular matrix raises as numpy.linalg.inv does."""
    from helpers import gpu_solver
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "c1_reference.npz")))
    s, _ = gpu_solver(synthetic_xs, 64, 1, False, 1)
    ff = g["ff"]
    out = s.normalized_distribution(0, 3.7 * ff)
    assert _rel(out, ff) <= 1e-12
    rng = np.random.default_rng(5)
    J = np.eye(40)[None] * 4.0 + rng.standard_normal((6, 40, 40))
    inv = s.batched_inv(0, J)
    assert _rel(inv, np.linalg.inv(J)) <= 1e-10
    J[2] = 0.0
    with pytest.raises(np.linalg.LinAlgError):
        s.batched_inv(0, J)


def test_compute_qoi_both_v_spaces(synthetic_xs):
    """compute_qoi of the FVM and the spectral 1D3V solvers against the reference's
    (tests/golden/qoi_1d3v_reference.npz)."""
    import ast
    from boltzmann_gb300.bte_1d3v import bte_1d3v
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    q = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi_1d3v_reference.npz")))
    f = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs))
    for k in ("v0", "vp"):
        out = f.compute_qoi(q["fvm_%s" % k], 0.0, 1e-3)
        for name in ("rates", "ne", "Te"):
            assert _rel(out[name].cpu().numpy(), q["fvm_%s_%s" % (k, name)]) <= 1e-12, (k, name)
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bte1d_reference.npz")))
    s = bte_1d3v(dict(ast.literal_eval(str(g["params"])), collisions=synthetic_xs))
    for k in ("v0", "v1", "v3"):
        out = s.compute_qoi(np.real(g[k]), 0.0, 1e-3)
        for name in ("rates", "ne", "Te"):
            assert _rel(out[name].cpu().numpy(), q["spec_%s_%s" % (k, name)]) <= 1e-11, (k, name)


def test_projections_and_radial_components(synthetic_xs):
    """ords_to_sph / sph_to_ords and compute_radial_components of both 1D3V solvers against the
    reference's (tests/golden/qoi_1d3v_reference.npz)."""
    import ast
    from boltzmann_gb300.bte_1d3v import bte_1d3v
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    q = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi_1d3v_reference.npz")))
    f = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs))
    U = f.ords_to_sph(q["fvm_vp"])
    assert _rel(U.cpu().numpy(), q["fvm_vp_sph"]) <= 1e-13
    assert f.sph_to_ords(U).shape == (f.dof_v, f.dof_x)
    assert _rel(f.compute_radial_components(q["ev"], q["fvm_vp"]), q["fvm_vp_radial"]) <= 1e-13
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bte1d_reference.npz")))
    s = bte_1d3v(dict(ast.literal_eval(str(g["params"])), collisions=synthetic_xs))
    assert _rel(s.compute_radial_components(q["ev"], np.real(g["v3"])), q["spec_v3_radial"]) <= 1e-11


def test_checkpoint_through_the_solver(synthetic_xs, tmp_path):
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    q = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi_1d3v_reference.npz")))
    f = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs))
    pre = str(tmp_path / "fvm_cp")
    f.store_checkpoint(q["fvm_vp"], 0.5, 1e-3, pre)
    t, dt, v = f.restore_checkpoint(pre)
    assert (t, dt) == (0.5, 1e-3) and np.array_equal(v.cpu().numpy(), q["fvm_vp"])
    with np.load(pre + ".npz") as F:
        assert _rel(F["ne[m^-3]"], q["fvm_vp_ne"]) <= 1e-12


def test_anisotropic_initial_state(synthetic_xs):
    """initialize(..., "anisotropic") through the library's Maxwellian against the reference's."""
    from helpers import gpu_solver
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "init_reference.npz")))
    s, _ = gpu_solver(synthetic_xs, 64, 1, False, 2)
    assert _rel(s.initialize(0, 2, "anisotropic"), g["anisotropic_64_1"]) <= 1e-12


def test_step_without_preconditioner(synthetic_xs, g):
    """pc_type "none": plain GMRES on rhs_mvec reaches the reference's step."""
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    s = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs, pc_type="none"))
    s.init(float(g["dt"]))
    y = s.step(g["E"], g["v0"], None, 0.0, float(g["dt"])).cpu().numpy()
    assert s.gmres_info["status"] == 0
    assert _rel(y, g["step"]) <= 1e-10


def test_normalize_edf_both_v_spaces(synthetic_xs):
    """normalize_edf: on the FVM grid against the reference's formula with its own mass
    functional; on the spectral grid, scale-invariant and consistent with compute_qoi's rates."""
    import ast
    from boltzmann_gb300.bte_1d3v import bte_1d3v
    from boltzmann_gb300.bte_1d3v_fvm import C_GAMMA, bte_1d3v_fvm
    q = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi_1d3v_reference.npz")))
    f = bte_1d3v_fvm(dict(PARAMS, collisions=synthetic_xs))
    v = q["fvm_vp"]
    want = v / ((q["fvm_op_mass"] @ v) * (2.0 * (f.bs_vth / C_GAMMA) ** 3))
    assert _rel(f.normalize_edf(v).cpu().numpy(), want) <= 1e-12
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "bte1d_reference.npz")))
    s = bte_1d3v(dict(ast.literal_eval(str(g["params"])), collisions=synthetic_xs))
    v3 = np.real(g["v3"])
    n1, n3 = s.normalize_edf(v3).cpu().numpy(), s.normalize_edf(3.0 * v3).cpu().numpy()
    assert _rel(n3, n1) <= 1e-13
