"""Golden vectors of the reference's finite-volume 1D3V set-up and op-split step, generated by
running the reference's own `bte_1d3v` (BESolver/python/bte_1d3v_solver.py) with the FVM
v-space on CPU.

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script. Small case: 12 Chebyshev
points, 8 B-splines (Nr = 7: 25 radial FVM cells), 8 ordinates, stencil orders 2, the
synthetic argon-like cross sections.

Harness steps, as the reference's own CPU use would need:
* `cusparse_spsolve` is CuPy-only and unbound here; `init()` builds its triangular solver
  only for the large-system path, so it is replaced by a stub. At this size the step uses the
  dense collision inverse PmatC.
* The dense upwind matrices are captured by wrapping the reference's `mesh.upwinded_dx` /
  `mesh.upwinded_dvt`. `init()` then edits the returned arrays in place: it zeroes the
  inflow rows and sets the v_r outflow entry. For v_theta it multiplies by
  diag(sin theta) afterwards (bte_1d3v_solver.py:1406-1452), which the fixture leaves to
  the test.
* The op-split step's three sweeps are CuPy raw kernels (rawkernel.py); they run here through
  `oracle/sweeps_oracle.py` (itself pinned to dense solves), so the fixture pins the step's
  composition: collision solve, layout swaps, inflow zeroing, coefficients and order
  (bte_1d3v_solver.py:1745-1870, type XVTVRC).

The fixture also keeps the collision operator on the FVM grid (op_col_en, from the reference's
`_Lop_eulerian_strong_form`, collision_operator_spherical.py:1334-1437) with the grid weights,
n0, np0 and the v-domain, from which the step's PmatC is built.

Writes `fvm_reference.npz`. Usage:  python tests/golden/make_golden_fvm.py
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

PARAMS = dict(G.PARAMS, vspace_type=0, Nr=7, Nvt=8, Np=12, pvr=2, pvt=2, px=2)


def _sweep(fn):
    def run(L, R, c1, c2, dt, b, out, nd, Nr, Nvt, Nx):
        out[...] = fn(np.asarray(L)[:nd], np.asarray(R)[:nd], np.asarray(c1), np.asarray(c2), dt, np.asarray(b), Nr,
                      Nvt, Nx).reshape(out.shape)
    return run


def main():
    tmp = tempfile.mkdtemp(prefix="fvm_golden_")
    xs = write_synthetic_lxcat(os.path.join(tmp, "eAr_golden.lxcat"))
    par = os.path.join(tmp, "bte1d.toml")
    G.write_toml(par, PARAMS, xs, os.path.join(tmp, "run"))
    cwd = os.getcwd()
    import_reference()
    import bte_1d3v_solver as S
    import mesh
    try:
        S.cusparse_spsolve = types.SimpleNamespace(SpSMSolver=lambda *a, **k: None)
        calls = []

        def wrap(name):
            f = getattr(mesh, name)

            def g(x, dorder, sw, direction, *a, **k):
                out = f(x, dorder, sw, direction, *a, **k)
                calls.append((name, len(x), direction, out))  # init() edits this array in place
                return out
            return g
        mesh.upwinded_dx, mesh.upwinded_dvt = wrap("upwinded_dx"), wrap("upwinded_dvt")
        S.cp_rk.adv_vr_BE = _sweep(SO.adv_vr_BE)
        S.cp_rk.adv_vt_BE = _sweep(SO.adv_vt_BE)
        S.cp_rk.adv_x_BE = _sweep(SO.adv_x_BE)

        b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
        p = b.params
        dt = p.dt
        b.init(dt)
        Nr, Nvt, Nx = b.dof_vr, b.dof_vt, b.dof_x
        v0 = np.asarray(b.initial_condition(0)).reshape(Nr * Nvt, Nx)
        E = G.efield(np.asarray(b.grid_info["x"]))
        y = np.asarray(b.step_op_split(E, np.copy(v0), None, 0.0, dt, S.pc_type.XVTVRC))
        def dense(name, n, direction):
            m = [c[3] for c in calls if c[0] == name and c[1] == n and c[2] == direction]
            assert len(m) == 1, (name, n, direction, len(m))
            return np.asarray(m[0])
        out = dict(
            Nr=Nr, Nvt=Nvt, Nx=Nx, pvr=p.pvr, pvt=p.pvt, px=p.px, dt=dt, tau=p.tau, L=p.L, qe=p.qe, me=p.me,
            vth=b.bs_vth, vr=np.asarray(b.grid_info["vr"]), vt=np.asarray(b.grid_info["vt"]),
            x=np.asarray(b.grid_info["x"]),
            vr_diag_l2r=np.asarray(b.vr_diag_l2r), vr_diag_r2l=np.asarray(b.vr_diag_r2l),
            vt_diag_l2r=np.asarray(b.vt_diag_l2r), vt_diag_r2l=np.asarray(b.vt_diag_r2l),
            x_diag_l2r=np.asarray(b.x_diag_l2r), x_diag_r2l=np.asarray(b.x_diag_r2l),
            Dvr_LtoR=dense("upwinded_dx", Nr, "L"), Dvr_RtoL=dense("upwinded_dx", Nr, "R"),
            Dx_LtoR=dense("upwinded_dx", Nx, "L"), Dx_RtoL=dense("upwinded_dx", Nx, "R"),
            Dvt_LtoR=dense("upwinded_dvt", Nvt, "L"), Dvt_RtoL=dense("upwinded_dvt", Nvt, "R"),
            PmatC=np.asarray(b.PmatC), v0=v0, E=E, step=y,
            op_col_en=np.asarray(b.op_col_en.toarray() if hasattr(b.op_col_en, "toarray") else b.op_col_en),
            vr_qw=np.asarray(b.grid_info["vr_qw"]), vt_qw=np.asarray(b.grid_info["vt_qw"]), n0=p.n0, np0=p.np0,
            domain=np.asarray(b.op_spec_sp._basis_p._domain, dtype=np.float64), spline_qpts=p.spline_qpts)
        assert Nr != Nx and Nr != Nvt and Nx != Nvt  # grids told apart by size
        np.savez_compressed(os.path.join(HERE, "fvm_reference.npz"), **{k: v for k, v in out.items()})
        print("wrote fvm_reference.npz: dof_v %d, Nx %d, |step| %.6e" % (Nr * Nvt, Nx, np.linalg.norm(y)))
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
