"""Golden vectors of the reference's semi-Lagrangian finite-volume 1D3V step, generated by running
the reference's own `bte_1d3v` (BESolver/python/bte_1d3v_solver.py) with `vspace_type = 0` and
`solver_type = "sl_implicit"` on CPU: the (v, x) advection by interpolation at the departure
points (`step_adv_vx_sl`, :2244-2314, SciPy `interpn` on the CPU path) followed by the collision
solve PmatC (:2024-2027).

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script. Same small grid as
`make_golden_fvm.py` (12 Chebyshev-Gauss-Lobatto x points, 25 radial cells, 8 ordinates), with
dt = 5e-3 periods and the field scaled up (peak ~1.8e5 V/m, both signs) so that the departure
points move by a sizeable part of a cell in x and in v and leave the domain at the inflow
boundary.

Writes `fvm_sl_reference.npz`. Usage:  python tests/golden/make_golden_fvm_sl.py
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
import make_golden_1d3v as G  # noqa: E402
import make_golden_fvm as GF  # noqa: E402

PARAMS = dict(GF.PARAMS, xspace_type=0, solver_type="sl_implicit", dt=5e-3)


def main():
    tmp = tempfile.mkdtemp(prefix="fvm_sl_golden_")
    xs = write_synthetic_lxcat(os.path.join(tmp, "eAr_golden.lxcat"))
    par = os.path.join(tmp, "bte1d.toml")
    G.write_toml(par, PARAMS, xs, os.path.join(tmp, "run"))
    cwd = os.getcwd()
    import_reference()
    import bte_1d3v_solver as S
    try:
        S.cusparse_spsolve = types.SimpleNamespace(SpSMSolver=lambda *a, **k: None)
        b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
        p = b.params
        dt = p.dt
        b.init(dt)
        Nr, Nvt, Nx = b.dof_vr, b.dof_vt, b.dof_x
        v0 = np.asarray(b.initial_condition(0)).reshape(Nr * Nvt, Nx)
        E = 50.0 * G.efield(np.asarray(b.grid_info["x"]))
        E[3] = -0.5 * abs(E[3])
        v_sl = np.asarray(b.step_adv_vx_sl(E, np.copy(v0), 0.0, dt))
        y = np.asarray(b.step(E, np.copy(v0), None, 0.0, dt))
        out = dict(
            Nr=Nr, Nvt=Nvt, Nx=Nx, dt=dt, tau=p.tau, L=p.L, qe=p.qe, me=p.me, n0=p.n0, np0=p.np0, vth=b.bs_vth,
            vr=np.asarray(b.grid_info["vr"]), vt=np.asarray(b.grid_info["vt"]), x=np.asarray(b.grid_info["x"]),
            kdomain=np.asarray(b.op_spec_sp._basis_p._kdomain, dtype=np.float64), PmatC=np.asarray(b.PmatC),
            v0=v0, E=E, v_sl=v_sl, step=y)
        np.savez_compressed(os.path.join(HERE, "fvm_sl_reference.npz"), **out)
        print("wrote fvm_sl_reference.npz: dof_v %d, Nx %d, |v_sl - v0| / |v0| %.3e, |step| %.6e"
              % (Nr * Nvt, Nx, np.linalg.norm(v_sl - v0) / np.linalg.norm(v0), np.linalg.norm(y)))
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
