"""Golden vectors of the 1D3V spectral step, generated by running the reference's own
`bte_1d3v` (BESolver/python/bte_1d3v_solver.py) on CPU.

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script. Small case: 16 Chebyshev
points, 16 B-splines (Nr = 15), l_max 1, 8 ordinates, BE Chebyshev x-space, spectral
v-space, the synthetic argon-like cross sections. Writes `bte1d_reference.npz`: the
reference's setup operators (Chebyshev derivative, ordinates, projections, radial
x-advection operator and eigenbasis, v-space operators) and one Strang step
(x over dt/2, v over dt with its GMRES, x over dt/2) from its initial condition at a
non-uniform field.

Two harness steps work around the reference's current spectral path, as its own drivers
would need: `__initialize_bte_adv_x__` builds the x-advection inverses only when the solver
type is "fully implicit" (bte_1d3v_solver.py:785-786), so it is called with that type set
for the call; the v-space preconditioner (PmatE, Evals) is built as init() does for the
spectral v-space (:1333-1344), because init() continues into FVM-only set-up.

Usage:  python tests/golden/make_golden_1d3v.py
"""
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from boltzmann_gb300.workloads import write_synthetic_lxcat  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402

PARAMS = dict(L=2.54e-2, V0=100.0, freq=13.56e6, Tg=300.0, p0=1.0, abs_efield_min=1e-6, abs_efield_max=1e3,
              num_pc_ops=16, vspace_ts_type="BE", atol=1e-14, rtol=1e-12, gmres_rsrt=30, gmres_rsrt_iter=20,
              max_iter=300, use_gpu=0, gpu_device_id=0, restore=0, rs_idx=0, ic_file="", fname="bte1d",
              plot_data=0, io_cycle=1.0, cp_cycle=1.0, threads=1, Np=16, Nr=15, Nvt=8, lmax=1, dt=1e-3,
              ev_max=80.0, ev_extend=0, sp_order=3, spline_qpts=5, Te=4.0, cycles=1, verbose=0,
              xspace_type=1, vspace_type=1, solver_type="xvx_strang_split", adaptive_grid=1)


def efield(xp):
    """Non-uniform field (V/m) on the Chebyshev points: the reference's v-step takes its GMRES
    path only when E varies over x (bte_1d3v_solver.py:1011)."""
    return 3.0e3 * (0.2 + xp) * (1.0 - 0.3 * xp ** 2)


def write_toml(path, params, collisions, run_dir):
    with open(path, "w") as fh:
        fh.write("[bte]\n")
        for k, v in dict(params, collisions=collisions, dir=run_dir).items():
            fh.write("%s = %s\n" % (k, ('"%s"' % v) if isinstance(v, str) else repr(v)))


def main():
    tmp = tempfile.mkdtemp(prefix="bte1d_golden_")
    xs = write_synthetic_lxcat(os.path.join(tmp, "eAr_golden.lxcat"))
    par = os.path.join(tmp, "bte1d.toml")
    write_toml(par, PARAMS, xs, os.path.join(tmp, "run"))
    cwd = os.getcwd()
    import_reference()
    import bte_1d3v_solver as S
    try:
        b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
        p = b.params
        dt = p.dt
        st = p.solver_type
        p.solver_type = S.solver_type.FULLY_IMPLICIT
        b.__initialize_bte_adv_x__(0.5 * dt)
        p.solver_type = st
        ep = np.logspace(np.log10(p.pcEmin), np.log10(p.pcEmax), p.pcN // 2, base=10)
        b.Evals = np.append(-np.flip(ep), ep)
        vmat = p.tau * p.n0 * p.np0 * (b.op_col_en + p.Tg * b.op_col_gT)
        Iv = np.eye(b.op_adv_v.shape[0])
        b.PmatE = np.array([np.linalg.inv(Iv - dt * p.tau * b.Evals[i] * b.op_adv_v - dt * p.tau * vmat)
                            for i in range(p.pcN)])
        v0 = np.asarray(b.initial_condition(0))
        E = efield(np.asarray(b.xp))
        v1 = np.asarray(b.step_bte_x(np.copy(v0), 0.0, 0.5 * dt))
        v2 = np.asarray(b.step_bte_v(E, np.copy(v1), None, 0.0, dt))
        v3 = np.asarray(b.step_bte_x(np.copy(v2), 0.5 * dt, 0.5 * dt))
        out = dict(params=np.array(repr(PARAMS)), xp=np.asarray(b.xp), Dp=np.asarray(b.Dp), xp_vt=b.xp_vt,
                   xp_vt_qw=b.xp_vt_qw, op_po2sh=b.op_po2sh, op_psh2o=b.op_psh2o, op_adv_x=b.op_adv_x,
                   op_adv_x_d=b.op_adv_x_d, op_col_en=b.op_col_en, op_col_gT=b.op_col_gT, op_adv_v=b.op_adv_v,
                   op_mass=b.op_mass, tau=p.tau, n0=p.n0, np0=p.np0, L=p.L, vth=b.bs_vth, E=E, v0=v0, v1=v1, v2=v2,
                   v3=v3)
        np.savez_compressed(os.path.join(HERE, "bte1d_reference.npz"), **out)
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
