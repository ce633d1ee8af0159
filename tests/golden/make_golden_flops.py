"""Golden values of the reference's flop model (`bte_0d3v_batched.rhs_and_jac_flops`,
BESolver/python/bte_0d3v_batched.py:823-854), generated by calling the reference's own class
(CPU path, one species, e-e off and on) at the bordered sizes of the configurations.

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script.
Writes `flops_reference.json`. Usage:  python tests/golden/make_golden_flops.py
"""
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from boltzmann_gb300.workloads import write_synthetic_lxcat, EV_MAX, TE_NORM  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402

CASES = [(n, p) for n in (128, 384, 1280) for p in (1, 7, 4096)]


def main():
    xs = write_synthetic_lxcat(os.path.join("/tmp", "eAr_flops.lxcat"))
    cwd = os.getcwd()
    m = import_reference()
    out = {}
    try:
        for ee in (0, 1):
            args = types.SimpleNamespace(threads=1, sp_order=3, spline_qpts=5, ee_collisions=ee, verbose=0, use_gpu=0,
                                         Efreq=0.0, dt=1e-3, cycles=1, solver_type="steady-state", l_max=1, Nr=63,
                                         n_pts=1, out_fname="/tmp/golden")
            s = m.bte_0d3v_batched(args, np.array([EV_MAX]), np.array([TE_NORM]), np.array([63]), [[[0, 0], [1, 0]]],
                                   1, [xs])
            res, jac = s.rhs_and_jac_flops()
            out["ee%d" % ee] = [[n, p, int(res(n, p)), int(jac(n, p))] for n, p in CASES]
    finally:
        os.chdir(cwd)
        os.unlink(xs)
    with open(os.path.join(HERE, "flops_reference.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote flops_reference.json")


if __name__ == "__main__":
    main()
