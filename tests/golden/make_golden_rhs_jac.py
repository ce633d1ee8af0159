"""Golden residuals, Jacobians and a transient step from the reference itself (CPU path).

Runs the reference's own `bte_0d3v_batched.get_rhs_and_jacobian` (BESolver/python/
bte_0d3v_batched.py:602-821) and `step` (:981-1032) on the e-e fixture's grid (16 B-splines,
l_max 2, 3 points) and records, at a fixed state x (the e-e-off steady state of each point,
mass-normalized, plus a seeded perturbation so that no term vanishes):
  * res_ee / jac_ee and res_noee / jac_noee: the projected residual (m, P) and Jacobian
    (P, m, m) with the e-e term on and off;
  * qmat: the reference's constraint basis Q (n, m), which both closures are taken against;
  * step_v: one backward-Euler step v = u + Q du of `step` from u = x with the chord
    iteration at atol 1e-30, rtol 1e-12, 50 iterations, time 0, delta_t 2e-10 s, e-e on.
Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script.

Usage:  python tests/golden/make_golden_rhs_jac.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from boltzmann_gb300.workloads import write_synthetic_lxcat, N0_1TORR_300K  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402
import make_golden as G  # noqa: E402


def main():
    xs = write_synthetic_lxcat(os.path.join("/tmp", "eAr_rhsjac_%d.lxcat" % os.getpid()))
    cwd = os.getcwd()
    m = import_reference()
    try:
        n_sp, l_max, P = 16, 2, 3
        s, args = G.make_solver(m, xs, n_sp, l_max, True, P)
        n0 = np.full(P, N0_1TORR_300K)
        prm = dict(n0=n0, ne=np.array([1e-5, 1e-4, 1e-3]) * n0, Tg=np.full(P, 300.0),
                   E=np.array([30.0, 100.0, 300.0]) * n0 * 1e-21, ns_by_n0=np.ones((1, P)))
        f0 = s.initialize(0, P, "maxwellian")
        G.set_params(s, prm)
        args.ee_collisions = 0
        ffw, _ = s.solve(0, f0, G.ATOL, G.RTOL, G.MAXIT, "steady-state", alpha_min=1e-16, alpha_rho=0.5,
                         line_search_c=1e-4)
        import utils as bte_utils
        vth = s._par_vth[0]
        u = s._op_mass[0] * bte_utils.get_maxwellian_3d(vth, 1)(0) * vth ** 3
        x = ffw / np.dot(u, ffw)
        rng = np.random.default_rng(11)
        x = x * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, x.shape))
        out = dict(n0=prm["n0"], ne=prm["ne"], Tg=prm["Tg"], E=prm["E"], ns_by_n0=prm["ns_by_n0"], x=x,
                   qmat=s._op_qmat[0], rmat=s._op_rmat[0])
        for ee in (0, 1):
            args.ee_collisions = ee
            res, jac = s.get_rhs_and_jacobian(0, P)
            tag = "ee" if ee else "noee"
            out["res_" + tag] = res(x, 0.0, 0.0)
            out["jac_" + tag] = jac(x, 0.0, 0.0)
        args.ee_collisions = 1
        args.Efreq = 13.56e6
        out["step_dt"] = 2e-10
        out["step_v"] = s.step(0, x, 1e-30, 1e-12, 50, 0.0, out["step_dt"])
        np.savez_compressed(os.path.join(HERE, "rhs_jac_reference.npz"), **out)
        print("wrote rhs_jac_reference.npz", {k: np.shape(v) for k, v in out.items()})
    finally:
        os.chdir(cwd)
        os.unlink(xs)


if __name__ == "__main__":
    main()
