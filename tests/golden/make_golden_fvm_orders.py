"""Golden FVM set-up of the reference's own `bte_1d3v` (BESolver/python/bte_1d3v_solver.py,
`vspace_type = 0`, `solver_type = "fully_implicit"`, upwind x) at stencil orders 1 and 3, on
CPU: the sweeps' six band arrays (:1403-1470), the v-space advection matrices for both field
signs (spec_spherical.py:876-951) and the x-shift bands (:780-860). Together with
`fvm_implicit_reference.npz` (order 2) they pin the oracle's upwind operators at every
stencil order the tests use.

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script.
Writes `fvm_orders_reference.npz`. Usage:  python tests/golden/make_golden_fvm_orders.py
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
import make_golden_fvm_implicit as GI  # noqa: E402

CASES = {1: dict(Nr=6, Nvt=6, Np=9), 3: dict(Nr=8, Nvt=10, Np=11)}


def main():
    tmp = tempfile.mkdtemp(prefix="fvm_orders_golden_")
    xs = write_synthetic_lxcat(os.path.join(tmp, "eAr_golden.lxcat"))
    cwd = os.getcwd()
    import_reference()
    import bte_1d3v_solver as S
    out = {}
    try:
        S.cusparse_spsolve = types.SimpleNamespace(SpSMSolver=lambda *a, **k: None)
        for p, sizes in CASES.items():
            par = os.path.join(tmp, "p%d.toml" % p)
            G.write_toml(par, dict(GI.PARAMS, pvr=p, pvt=p, px=p, **sizes), xs, os.path.join(tmp, "run%d" % p))
            b = S.bte_1d3v(types.SimpleNamespace(par_file=par))
            b.init(b.params.dt)
            pre = "p%d_" % p
            out.update({pre + k: np.asarray(getattr(b, k)) for k in ("vr_diag_l2r", "vr_diag_r2l", "vt_diag_l2r",
                                                                    "vt_diag_r2l", "x_diag_l2r", "x_diag_r2l",
                                                                    "op_adv_v_Ep", "op_adv_v_En", "bte_x_shift_diag")})
            out.update({pre + "vr": np.asarray(b.grid_info["vr"]), pre + "vt": np.asarray(b.grid_info["vt"]),
                        pre + "x": np.asarray(b.grid_info["x"]),
                        pre + "domain": np.asarray(b.op_spec_sp._basis_p._domain, dtype=np.float64),
                        pre + "dt": b.params.dt, pre + "ax": b.bs_vth * b.params.tau / b.params.L,
                        pre + "cA": b.params.qe / b.params.me / b.bs_vth})
        np.savez_compressed(os.path.join(HERE, "fvm_orders_reference.npz"), **out)
        print("wrote fvm_orders_reference.npz")
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
