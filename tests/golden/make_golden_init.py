"""Golden initial states of the reference's `bte_0d3v_batched.initialize`
(BESolver/python/bte_0d3v_batched.py:481-520), "maxwellian" and "anisotropic" (a Maxwellian
times 1 + cos(theta)), from the reference's own class on CPU, for 64 B-splines with l_max 1
and 16 B-splines with l_max 2 (the grids of the c1 and e-e fixtures).

Runs only where the reference checkout is available (imported through
`oracle/reference_import.py`); the GPU host never runs this script.
Writes `init_reference.npz`. Usage:  python tests/golden/make_golden_init.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from boltzmann_gb300.workloads import write_synthetic_lxcat  # noqa: E402
from oracle.reference_import import import_reference  # noqa: E402
import make_golden as G  # noqa: E402


def main():
    xs = write_synthetic_lxcat(os.path.join("/tmp", "eAr_init.lxcat"))
    cwd = os.getcwd()
    m = import_reference()
    out = {}
    try:
        for n_sp, l_max in ((64, 1), (16, 2)):
            s, _ = G.make_solver(m, xs, n_sp, l_max, False, 1)
            for kind in ("maxwellian", "anisotropic"):
                out["%s_%d_%d" % (kind, n_sp, l_max)] = np.asarray(s.initialize(0, 2, kind))
    finally:
        os.chdir(cwd)
        os.unlink(xs)
    np.savez_compressed(os.path.join(HERE, "init_reference.npz"), **out)
    print("wrote init_reference.npz:", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
