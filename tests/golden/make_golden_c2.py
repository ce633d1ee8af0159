"""Golden EDFs at the benchmarked shapes, from the reference itself (CPU path).

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script. It writes:

  c2_shape_reference.npz   128 B-splines, l_max 2 (n = 384, the batched workload's grid),
                           e-e on, 8 points. Three of them sit at E/N < 10 Td with an
                           ionization degree above 1e-4, where the Coulomb term dominates.
  c5_reduced_reference.npz 64 B-splines, l_max 4 (n = 320, the large workload's angular
                           resolution on a coarser radial grid), e-e on, 4 points with
                           ionization degrees in [1e-6, 1e-2].

Each solve follows the reference driver (`BESolver/python/bte_0d3v_batched_driver.py:192-204`):
Maxwellian -> e-e-off solve -> e-e-on solve from that result, with atol 1e-20, rtol 1e-14,
100 iterations, alpha_rho 0.5, c 1e-4. Besides the EDFs and QoIs, the fixture records each
point's final residual norm of the e-e-on phase and its ratio to the phase's initial norm,
evaluated with the reference's own `get_rhs_and_jacobian` residual
(`BESolver/python/bte_0d3v_batched.py:602-821`) at the state the solve stopped at, so a test
can tell a converged point from one where the reference stopped at its line-search break
(`:947-956`).

With --perturbed (run after the plain run), the same solves are repeated with the
reference's operators perturbed at the rounding level (4 ulps, seeded), and the fixture gains
`ff_perturbed` and `resolution`, the per-point relative L2 shift of the EDF: how precisely
FP64 arithmetic determines the reference's own answer at that point.

With --perturbed-mass, the perturbation is one rounding unit on each mass-matrix entry,
carried through the reference's M^-1 scaling of its operators; the fixture gains
`ff_perturbed_mass` and `resolution_mass`.

With --swap-rosenbluth=FILE (one fixture; FILE from export_device_rosenbluth.py on a GPU host,
for that fixture's grid), the reference's Coulomb operator is rebuilt from its own trilinear
tensors and the device library's Rosenbluth potentials and the points are solved again by the
reference; the fixture gains `ff_device_rosenbluth` and `rosenbluth_swap_shift`.

With --exact (after the plain run), `exact()` below adds the exact fixed points of the
reference's own discrete systems: `ff_warm_exact`, `ff_exact`, `warm_exact_shift`, `exact_shift`;
with --exact --swap-rosenbluth=FILE (after --swap-rosenbluth), the e-e-on fixed point of the
system built with the device potentials: `ff_exact_device_rosenbluth`.

Usage:  python tests/golden/make_golden_c2.py [c2|c5] [--perturbed | --perturbed-mass | --swap-rosenbluth=FILE | --exact]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from boltzmann_gb300.workloads import write_synthetic_lxcat, N0_1TORR_300K, TD  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402
import make_golden as G  # noqa: E402

# (E/N in Td, ionization degree): the first three are the low-field, strongly ionized points.
C2_POINTS = [(1.5, 5e-4), (3.0, 2e-4), (7.0, 8e-4), (2.0, 1e-7), (30.0, 1e-5), (100.0, 1e-3),
             (400.0, 1e-6), (950.0, 3e-4)]
C5_POINTS = [(1.2, 8e-3), (20.0, 1e-6), (150.0, 1e-4), (700.0, 1e-2)]


def _state_of(s, ff):
    """The solver's unknown h for a normalized EDF: rescaled so that u.h = 1 (the constraint
    the reference's Newton iterates satisfy, bte_0d3v_batched.py:907-917)."""
    import utils as bte_utils
    vth = s._par_vth[0]
    mw = bte_utils.get_maxwellian_3d(vth, 1)
    qA = s._op_diag_dg[0]
    u = np.dot(np.transpose(s._op_mass[0] * mw(0) * vth ** 3), qA)
    h = np.dot(qA.T, ff / np.dot(u, ff))
    return h, u


def _initial_state(s, f0):
    """h_prev of steady_state_solve's first iteration (bte_0d3v_batched.py:907-917)."""
    h, u = _state_of(s, f0)
    f1 = u / np.dot(u, u)
    return f1[:, None] + np.dot(s._op_qmat[0], np.dot(s._op_rmat[0], h))


def _perturb(s, seed, ulps=4.0):
    """Multiply every entry of the reference's assembled collision, gas-temperature, advection
    and Coulomb operators by (1 + ulps * eps * u), u uniform in [-1, 1]: a change smaller than
    the rounding any FP64 assembly of those operators carries (quadrature sums, the Cholesky
    inverse of the mass matrix)."""
    rng = np.random.default_rng(seed)
    eps = np.finfo(np.float64).eps
    for name in ("_op_col_en", "_op_col_gT", "_op_advection", "_op_col_ee"):
        op = getattr(s, name)[0]
        if op is None or np.ndim(op) == 0:
            continue
        getattr(s, name)[0] = op * (1.0 + ulps * eps * rng.uniform(-1.0, 1.0, np.shape(op)))


def _perturb_mass(s, seed):
    """Change the mass matrix by one rounding unit per entry (symmetric, seeded) and carry it
    through the reference's M^-1 scaling of every operator, to first order:
    op <- op - M^-1 (dM op). The reference's operators are M^-1 times raw integrals, and M^-1
    inherits the mass matrix's conditioning; this is the size of perturbation that any FP64
    assembly of M (a quadrature sum) leaves in them."""
    rng = np.random.default_rng(seed)
    eps = np.finfo(np.float64).eps
    M = s._op_mass_mat[0]
    u = rng.uniform(-1.0, 1.0, M.shape)
    dM = eps * np.abs(M) * np.triu(u) + (eps * np.abs(M) * np.triu(u, 1)).T
    Minv = s._op_spec_sp[0].inverse_mass_mat(Mmat=M)
    for name in ("_op_col_en", "_op_col_gT", "_op_advection", "_op_col_ee"):
        op = getattr(s, name)[0]
        if op is None or np.ndim(op) == 0:
            continue
        if name == "_op_col_en":  # (species, n, n)
            new = np.stack([o - Minv @ (dM @ o) for o in op])
        else:                     # (n, n) or (n, n, n): M^-1 acts on the first index
            flat = op.reshape(op.shape[0], -1)
            new = (flat - Minv @ (dM @ flat)).reshape(op.shape)
        getattr(s, name)[0] = new


def _swap_rosenbluth(s, path):
    """Rebuild the reference's Coulomb operator from its own trilinear tensors and the device
    library's Rosenbluth potentials (export_device_rosenbluth.py), as assemble_operators builds
    it (bte_0d3v_batched.py:444-476: M^-1 (cc_a . hl + cc_b . gl), qA = I)."""
    import collision_operator_spherical as cos
    import utils
    d = np.load(path)
    spec = s._op_spec_sp[0]
    mw = utils.get_maxwellian_3d(s._par_vth[0], 1)
    cca, ccb = cos.CollisionOpSP(spec).coulomb_collision_op_assembly(mw, s._par_vth[0], mp_pool_sz=1)
    n = cca.shape[0]
    Minv = spec.inverse_mass_mat(Mmat=s._op_mass_mat[0])
    cc = np.dot(cca, d["hl"]) + np.dot(ccb, d["gl"])
    s._op_col_ee[0] = np.dot(Minv, cc.reshape((n, -1))).reshape((n, n, n))


def exact(m, xs, name, n_sp, l_max, iters=6, swap=None):
    """The exact fixed points of the reference's own discrete systems at the fixture's points,
    for both phases of the driver sequence (e-e off: `ff_warm`, e-e on: `ff`).

    The reference's Newton (bte_0d3v_batched.py:882-979) uses a Jacobian without two rank-one
    terms: the derivative of the growth term's scalar n0 sum_s ns W x and of the Coulomb
    logarithm (its dgamma_a_df term, :663, is commented out at :750-751 of jac_func). It
    therefore converges linearly, and where the e-e term dominates its FP64 residual reaches
    its rounding floor before the iterate reaches the fixed point. Here the reference's own
    residual closure is evaluated in extended precision (np.longdouble, the operators being
    the reference's FP64 arrays), and Newton corrections with the full Jacobian (the
    reference's jac_func plus the rank-one terms, FP64 solves) start from the reference's
    stopped solution. The fixture gains `ff_exact` / `ff_warm_exact`, `exact_shift` /
    `warm_exact_shift` (the reference's own distance from that fixed point, relative L2) and
    `exact_steps` / `warm_exact_steps` (the size of the last correction).

    With `swap` (the device library's Rosenbluth potentials, as for --swap-rosenbluth), the
    e-e-on fixed point of the reference's system built with those potentials is computed from
    the reference's answer with them (`ff_device_rosenbluth`): `ff_exact_device_rosenbluth`."""
    import utils as bte_utils
    import scipy.constants as sc
    g = dict(np.load(os.path.join(HERE, name)))
    P = g["ff"].shape[1]
    s, args = G.make_solver(m, xs, n_sp, l_max, True, P)
    if swap is not None:
        _swap_rosenbluth(s, swap)
    G.set_params(s, {k: g[k] for k in ("n0", "ne", "Tg", "E", "ns_by_n0")})
    Q = s._op_qmat[0]
    vth = s._par_vth[0]
    mw = bte_utils.get_maxwellian_3d(vth, 1)
    u = s._op_mass[0] * mw(0) * vth ** 3
    Wmat = np.einsum("v,svu->su", u, s._op_col_en[0])
    c_ee = s._op_col_ee[0]
    Mop, Top = s._op_mass[0], s._op_temp[0]
    gam_c = sc.e ** 4 / (4 * np.pi * (sc.epsilon_0 * sc.electron_mass) ** 2) / vth ** 3
    w = (g["n0"] * g["ns_by_n0"]).T @ Wmat  # (P, n): gradient of the growth term's scalar
    phases = ((0, "ff_warm", "warm_exact"), (1, "ff", "exact"))
    if swap is not None:
        phases = ((1, "ff_device_rosenbluth", "exact_device_rosenbluth"),)
    for ee, key, out in phases:
        args.ee_collisions = ee
        res_func, jac_func = s.get_rhs_and_jacobian(0, P)
        h, _ = _state_of(s, g[key])
        hl = h.astype(np.longdouble)
        Ql = Q.astype(np.longdouble)
        steps = None
        for it in range(iters):
            r = res_func(hl, 0, 0)
            x = hl.astype(np.float64)
            L = jac_func(x, 0, 0)
            qx = Q.T @ x
            if ee:
                qc = Q.T @ np.einsum("abc,bc->ac", np.dot(c_ee, x), x)
                tx, mx = Top @ x, Mop @ x
            for a in range(P):
                L[a] = L[a] - np.outer(qx[:, a], Q.T @ w[a])
                if ee:  # gradient of the Coulomb logarithm factor
                    grad = gam_c * 1.5 * (Top / tx[a] - Mop / mx[a])
                    L[a] = L[a] + g["ne"][a] * np.outer(qc[:, a], Q.T @ grad)
            pp = np.linalg.solve(L, -np.asarray(r, dtype=np.float64).T[..., None])[..., 0].T
            hl = hl + Ql @ pp.astype(np.longdouble)
            steps = np.linalg.norm(pp, axis=0) / np.linalg.norm(h, axis=0)
            print("%s %s: correction %d %s" % (name, out, it, np.array2string(steps, precision=2)), flush=True)
        ffx = s.normalized_distribution(0, hl.astype(np.float64))
        g[(key + "_exact") if swap is None else "ff_exact_device_rosenbluth"] = ffx
        g[out + "_shift"] = np.linalg.norm(g[key] - ffx, axis=0) / np.linalg.norm(ffx, axis=0)
        g[out + "_steps"] = steps
        print("%s: the reference's distance from the exact fixed point (%s) %s" % (
            name, key, np.array2string(g[out + "_shift"], precision=2)), flush=True)
    np.savez_compressed(os.path.join(HERE, name), **g)


def run(m, xs, name, n_sp, l_max, points, perturb_seed=None, mode="ulps", swap=None):
    P = len(points)
    t0 = time.time()
    s, args = G.make_solver(m, xs, n_sp, l_max, True, P)
    if perturb_seed is not None:
        (_perturb_mass if mode == "mass" else _perturb)(s, perturb_seed)
    if swap is not None:
        _swap_rosenbluth(s, swap)
    t_setup = time.time() - t0
    ebyn = np.array([p[0] for p in points])
    ion = np.array([p[1] for p in points])
    n0 = np.full(P, N0_1TORR_300K)
    prm = dict(n0=n0, ne=ion * n0, Tg=np.full(P, 300.0), E=ebyn * n0 * TD, ns_by_n0=np.ones((1, P)))
    f0 = s.initialize(0, P, "maxwellian")
    G.set_params(s, prm)
    args.ee_collisions = 0
    t1 = time.time()
    ffw, _ = s.solve(0, f0, G.ATOL, G.RTOL, G.MAXIT, "steady-state", alpha_min=1e-16, alpha_rho=0.5,
                     line_search_c=1e-4)
    args.ee_collisions = 1
    t2 = time.time()
    ff, qoi = s.solve(0, ffw, G.ATOL, G.RTOL, G.MAXIT, "steady-state", alpha_min=1e-16, alpha_rho=0.5,
                      line_search_c=1e-4)
    t3 = time.time()
    res_func, _ = s.get_rhs_and_jacobian(0, P)
    r0 = np.linalg.norm(res_func(_initial_state(s, ffw), 0, 0), axis=0)
    hf, _ = _state_of(s, ff)
    r1 = np.linalg.norm(res_func(hf, 0, 0), axis=0)
    if swap is not None:
        g = dict(np.load(os.path.join(HERE, name)))
        g["ff_device_rosenbluth"] = ff
        g["rosenbluth_swap_shift"] = np.linalg.norm(ff - g["ff"], axis=0) / np.linalg.norm(g["ff"], axis=0)
        np.savez_compressed(os.path.join(HERE, name), **g)
        print("%s: shift with the device potentials %s" % (name, np.array2string(g["rosenbluth_swap_shift"],
                                                                                  precision=2)), flush=True)
        return
    if perturb_seed is not None:
        # a second solve of the same points with operators perturbed at the rounding level:
        # how far the reference's own answer moves under FP64-level changes of its operators
        g = dict(np.load(os.path.join(HERE, name)))
        sfx = "_mass" if mode == "mass" else ""
        g["ff_perturbed" + sfx] = ff
        g["resolution" + sfx] = np.linalg.norm(ff - g["ff"], axis=0) / np.linalg.norm(g["ff"], axis=0)
        np.savez_compressed(os.path.join(HERE, name), **g)
        print("%s: resolution%s %s" % (name, sfx, np.array2string(g["resolution" + sfx], precision=2)), flush=True)
        return
    out = dict(n_sp=n_sp, l_max=l_max, EbyN=ebyn, ion_deg=ion, f0=f0, ff_warm=ffw, ff=ff,
               energy=qoi["energy"], mobility=qoi["mobility"], diffusion=qoi["diffusion"], rates=qoi["rates"],
               abs_error=r1, rel_error=r1 / r0, setup_s=t_setup, solve_s=np.array([t2 - t1, t3 - t2]), **prm)
    np.savez_compressed(os.path.join(HERE, name), **out)
    print("wrote %s: setup %.0f s, solves %.0f s + %.0f s, rel_error %s" %
          (name, t_setup, t2 - t1, t3 - t2, np.array2string(r1 / r0, precision=2)), flush=True)


def main():
    which = [w for w in sys.argv[1:] if not w.startswith("--")] or ["c2", "c5"]
    seed = 7 if ("--perturbed" in sys.argv or "--perturbed-mass" in sys.argv) else None
    mode = "mass" if "--perturbed-mass" in sys.argv else "ulps"
    swap = next((a.split("=", 1)[1] for a in sys.argv if a.startswith("--swap-rosenbluth=")), None)
    if swap is not None:
        swap = os.path.abspath(swap)
        if len(which) != 1:
            raise SystemExit("--swap-rosenbluth takes one fixture (c2 or c5): the potentials are per grid")
    xs = write_synthetic_lxcat(os.path.join("/tmp", "eAr_golden_%d.lxcat" % os.getpid()))
    cwd = os.getcwd()
    m = import_reference()
    try:
        if "--exact" in sys.argv:
            if "c2" in which:
                exact(m, xs, "c2_shape_reference.npz", 128, 2, swap=swap)
            if "c5" in which:
                exact(m, xs, "c5_reduced_reference.npz", 64, 4, swap=swap)
            return
        if "c2" in which:
            run(m, xs, "c2_shape_reference.npz", 128, 2, C2_POINTS, seed, mode, swap)
        if "c5" in which:
            run(m, xs, "c5_reduced_reference.npz", 64, 4, C5_POINTS, seed, mode, swap)
    finally:
        os.chdir(cwd)
        os.unlink(xs)


if __name__ == "__main__":
    main()
