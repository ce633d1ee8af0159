"""Generate golden vectors by running the reference itself (ut-padas/boltzmann, CPU path).

Runs only where the reference checkout is available (it imports it through
`oracle/reference_import.py`); the GPU host never runs this script. Writes
compressed .npz fixtures next to this file:

  c1_reference.npz      config c1 (64 B-splines, l_max 1, 100 Td, e-e off, 1 point):
                        the reference's M^-1-scaled operators, raw mass matrix, QoI
                        functionals, Maxwellian initial state, converged EDF and QoIs.
  ee_small_reference.npz  16 B-splines, l_max 2, e-e on, 3 points: the Coulomb trilinear
                        tensors (sparse), Rosenbluth operators, warm-started converged EDFs
                        and QoIs.
  transient_reference.npz 32 B-splines, l_max 1, 2 points, one RF period of the transient
                        solve at dt = 0.05 period: final state and cycle-averaged QoIs.

Usage:  python tests/golden/make_golden.py
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from boltzmann_gb300.workloads import write_synthetic_lxcat, config_parameters, N0_1TORR_300K, EV_MAX, TE_NORM  # noqa
from oracle.reference_import import import_reference  # noqa

ATOL, RTOL, MAXIT = 1e-20, 1e-14, 100


def make_solver(m, xs, n_sp, l_max, ee, n_pts):
    args = types.SimpleNamespace(threads=1, sp_order=3, spline_qpts=5, ee_collisions=int(ee), verbose=0, use_gpu=0,
                                 Efreq=0.0, dt=1e-3, cycles=1, solver_type="steady-state", l_max=l_max, Nr=n_sp - 1,
                                 n_pts=n_pts, out_fname="/tmp/golden")
    s = m.bte_0d3v_batched(args, np.array([EV_MAX]), np.array([TE_NORM]), np.array([n_sp - 1]),
                           [[[l, 0] for l in range(l_max + 1)]], 1, [xs])
    s.assemble_operators(0, vspace_ext=m.vspace_grid_extension.NONE)
    return s, args


def set_params(s, prm):
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, prm[k])


def c1(m, xs):
    s, args = make_solver(m, xs, 64, 1, False, 1)
    prm = config_parameters("c1", 1)
    f0 = s.initialize(0, 1, "maxwellian")
    set_params(s, prm)
    ff, qoi = s.solve(0, f0, ATOL, RTOL, MAXIT, "steady-state", alpha_min=1e-16, alpha_rho=0.5, line_search_c=1e-4)
    out = dict(
        n0=prm["n0"], ne=prm["ne"], Tg=prm["Tg"], E=prm["E"], ns_by_n0=prm["ns_by_n0"],
        knots=s._op_spec_sp[0]._basis_p._t, mass_mat=s._op_mass_mat[0], advection=s._op_advection[0],
        col_en=s._op_col_en[0], col_gT=s._op_col_gT[0], mass_op=s._op_mass[0], temp_op=s._op_temp[0],
        mobility_op=s._op_mobility[0], diffusion_op=s._op_diffusion[0], rate_op=np.array(s._op_rate[0]),
        qmat=s._op_qmat[0], f0=f0, ff=ff, energy=qoi["energy"], mobility=qoi["mobility"],
        diffusion=qoi["diffusion"], rates=qoi["rates"])
    np.savez_compressed(os.path.join(HERE, "c1_reference.npz"), **out)


def ee_small(m, xs):
    import collision_operator_spherical as cos
    import utils
    n_sp, l_max, P = 16, 2, 3
    s, args = make_solver(m, xs, n_sp, l_max, True, P)
    n0 = np.full(P, N0_1TORR_300K)
    prm = dict(n0=n0, ne=np.array([1e-5, 1e-4, 1e-3]) * n0, Tg=np.full(P, 300.0),
               E=np.array([30.0, 100.0, 300.0]) * n0 * 1e-21, ns_by_n0=np.ones((1, P)))
    spec = s._op_spec_sp[0]
    mw = utils.get_maxwellian_3d(s._par_vth[0], 1)
    cop = cos.CollisionOpSP(spec)
    cca, ccb = cop.coulomb_collision_op_assembly(mw, s._par_vth[0], mp_pool_sz=1)
    f0 = s.initialize(0, P, "maxwellian")
    set_params(s, prm)
    args.ee_collisions = 0
    ffw, _ = s.solve(0, f0, ATOL, RTOL, MAXIT, "steady-state", alpha_min=1e-16, alpha_rho=0.5, line_search_c=1e-4)
    args.ee_collisions = 1
    ff, qoi = s.solve(0, ffw, ATOL, RTOL, MAXIT, "steady-state", alpha_min=1e-16, alpha_rho=0.5,
                      line_search_c=1e-4)
    ia, ib = np.nonzero(cca), np.nonzero(ccb)
    out = dict(
        n0=prm["n0"], ne=prm["ne"], Tg=prm["Tg"], E=prm["E"], ns_by_n0=prm["ns_by_n0"],
        cc_a_idx=np.array(ia, dtype=np.int32), cc_a_val=cca[ia], cc_b_idx=np.array(ib, dtype=np.int32),
        cc_b_val=ccb[ib], col_ee=s._op_col_ee[0], ff_warm=ffw, ff=ff, energy=qoi["energy"],
        mobility=qoi["mobility"], diffusion=qoi["diffusion"], rates=qoi["rates"])
    np.savez_compressed(os.path.join(HERE, "ee_small_reference.npz"), **out)


def transient(m, xs):
    """solve(..., "transient") of the reference (bte_0d3v_batched.py:1063-1155): 32 B-splines,
    l_max 1, e-e off, 2 points driven at 13.56 MHz, dt = 0.05 RF period over one period."""
    n_sp, l_max, P = 32, 1, 2
    s, args = make_solver(m, xs, n_sp, l_max, False, P)
    args.dt, args.cycles, args.Efreq, args.solver_type = 0.05, 1.0, 13.56e6, "transient"
    n0 = np.full(P, N0_1TORR_300K)
    prm = dict(n0=n0, ne=np.zeros(P), Tg=np.full(P, 300.0), E=np.array([50.0, 200.0]) * n0 * 1e-21,
               ns_by_n0=np.ones((1, P)))
    eRe, eIm = np.array([120.0, 400.0]) * n0 * 1e-21, np.array([30.0, -100.0]) * n0 * 1e-21
    f0 = s.initialize(0, P, "maxwellian")
    set_params(s, prm)
    s.set_boltzmann_parameter(0, "eRe", eRe)
    s.set_boltzmann_parameter(0, "eIm", eIm)
    u, qoi = s.solve(0, f0, 1e-30, 1e-10, 200, "transient")
    out = dict(n0=prm["n0"], ne=prm["ne"], Tg=prm["Tg"], E=prm["E"], ns_by_n0=prm["ns_by_n0"], eRe=eRe, eIm=eIm,
               dt=args.dt, cycles=args.cycles, Efreq=args.Efreq, f0=f0, u=np.asarray(u), energy=qoi["energy"],
               mobility=qoi["mobility"], diffusion=qoi["diffusion"], rates=qoi["rates"])
    np.savez_compressed(os.path.join(HERE, "transient_reference.npz"), **out)


def main():
    xs = write_synthetic_lxcat(os.path.join("/tmp", "eAr_golden.lxcat"))
    cwd = os.getcwd()
    m = import_reference()
    try:
        c1(m, xs)
        ee_small(m, xs)
        transient(m, xs)
    finally:
        os.chdir(cwd)
        os.unlink(xs)


if __name__ == "__main__":
    main()
