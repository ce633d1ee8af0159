"""Golden vectors of the reference's fully implicit finite-volume 1D3V step, generated by running
the reference's own `bte_1d3v` (BESolver/python/bte_1d3v_solver.py) with `vspace_type = 0`,
`xspace_type = 0` (upwind x), `solver_type = "fully_implicit"` and the op-split (XVTVRC)
preconditioner on CPU.

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script. Same small case as
`make_golden_fvm.py`: 12 Chebyshev-Gauss-Lobatto x points, 8 B-splines (25 radial cells),
8 ordinates, stencil orders 2, the synthetic argon-like cross sections.

Harness steps, beyond those of `make_golden_fvm.py`:
* the x-advection matvec `cp_rk.banded_tri_mv_batched` (a CuPy raw kernel) runs through
  `oracle/sweeps_oracle.py`;
* the reference's `bte_utils.gmres` is wrapped to record the operator and the preconditioner
  it is handed (`rhs_mvec`, :1915-1955, and the op-split step, :1966) applied to a seeded
  vector, then runs unchanged.

Writes `fvm_implicit_reference.npz`. Usage:  python tests/golden/make_golden_fvm_implicit.py
"""
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from boltzmann_gb300.workloads import write_synthetic_lxcat  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402
from oracle import sweeps_oracle as SO  # noqa: E402
import make_golden_1d3v as G  # noqa: E402
import make_golden_fvm as GF  # noqa: E402

PARAMS = dict(GF.PARAMS, xspace_type=0, solver_type="fully_implicit", rtol=1e-12, atol=1e-14)


def main():
    tmp = tempfile.mkdtemp(prefix="fvm_implicit_golden_")
    xs = write_synthetic_lxcat(os.path.join(tmp, "eAr_golden.lxcat"))
    par = os.path.join(tmp, "bte1d.toml")
    G.write_toml(par, PARAMS, xs, os.path.join(tmp, "run"))
    cwd = os.getcwd()
    import_reference()
    import bte_1d3v_solver as S
    try:
        S.cusparse_spsolve = types.SimpleNamespace(SpSMSolver=lambda *a, **k: None)
        S.cp_rk.adv_vr_BE = GF._sweep(SO.adv_vr_BE)
        S.cp_rk.adv_vt_BE = GF._sweep(SO.adv_vt_BE)
        S.cp_rk.adv_x_BE = GF._sweep(SO.adv_x_BE)
        # the CuPy kernel computes in double whatever the input's type (SciPy's operator probes its
        # matvec with an integer vector to pick the operator's dtype)
        S.cp_rk.banded_tri_mv_batched = lambda diags, b, lower, *a, **k: SO.banded_tri_mv(
            np.asarray(diags, dtype=np.float64), np.asarray(b, dtype=np.float64), lower)
        seen = {}
        real_gmres = S.bte_utils.gmres

        def gmres(xp, A, b, *a, **k):
            u = np.random.default_rng(7).standard_normal(A.shape[0])
            seen.update(b=np.copy(b), u=u, Au=np.copy(A.matvec(np.copy(u))), Mu=np.copy(k["M"].matvec(np.copy(u))))
            return real_gmres(xp, A, b, *a, **k)
        S.bte_utils.gmres = gmres

        b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
        p = b.params
        dt = p.dt
        b.init(dt)
        Nr, Nvt, Nx = b.dof_vr, b.dof_vt, b.dof_x
        v0 = np.asarray(b.initial_condition(0)).reshape(Nr * Nvt, Nx)
        E = G.efield(np.asarray(b.grid_info["x"]))
        E[3] = -0.5 * abs(E[3])   # both field signs: the v-advection switches operators with sign(E)
        y = np.asarray(b.step(E, np.copy(v0), None, 0.0, dt))
        info = b.gmres_info
        out = dict(
            Nr=Nr, Nvt=Nvt, Nx=Nx, pvr=p.pvr, pvt=p.pvt, px=p.px, dt=dt, tau=p.tau, L=p.L, qe=p.qe, me=p.me,
            n0=p.n0, np0=p.np0, Tg=p.Tg, vth=b.bs_vth, rtol=p.rtol, atol=p.atol,
            vr=np.asarray(b.grid_info["vr"]), vt=np.asarray(b.grid_info["vt"]), x=np.asarray(b.grid_info["x"]),
            domain=np.asarray(b.op_spec_sp._basis_p._domain, dtype=np.float64),
            adv_v_Ep=np.asarray(b.op_adv_v_Ep), adv_v_En=np.asarray(b.op_adv_v_En),
            x_shift_diag=np.asarray(b.bte_x_shift_diag),
            v0=v0, E=E, step=y, brhs=seen["b"], u=seen["u"], Au=seen["Au"], Mu=seen["Mu"],
            gmres_residual_rel=float(info["residual_rel"]))
        np.savez_compressed(os.path.join(HERE, "fvm_implicit_reference.npz"), **out)
        print("wrote fvm_implicit_reference.npz: dof_v %d, Nx %d, |step| %.6e, rel. residual %.3e"
              % (Nr * Nvt, Nx, np.linalg.norm(y), info["residual_rel"]))
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
