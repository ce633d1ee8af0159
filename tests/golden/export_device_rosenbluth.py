"""Export the library's assembled Rosenbluth-potential operators (HL, GL) of a fixture's grid
(default the c2 shape, 128 B-splines and l_max 2; the reduced c5 fixture is 64 and 4) to an
.npz file, for make_golden_c2.py --swap-rosenbluth.

Runs on a GPU host with the library built. The swap experiment rebuilds the reference's Coulomb
operator from the reference's own trilinear tensors and these device potentials, and solves
again with the reference, to separate how much of the difference between the device solution
and the reference's comes from the potentials alone.

Usage:  python tests/golden/export_device_rosenbluth.py OUT.npz [N_SP L_MAX]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..")))

from helpers import gpu_solver  # noqa: E402
from boltzmann_gb300.workloads import write_synthetic_lxcat  # noqa: E402


def main(out, n_sp=128, l_max=2):
    xs = write_synthetic_lxcat()
    try:
        s, _ = gpu_solver(xs, n_sp, l_max, True, 1, "fp64")
        np.savez_compressed(out, hl=s.export_operator(0, "HL").cpu().numpy(),
                            gl=s.export_operator(0, "GL").cpu().numpy(),
                            minv=s.export_operator(0, "MINV").cpu().numpy())
    finally:
        os.unlink(xs)


if __name__ == "__main__":
    main(sys.argv[1], *(int(a) for a in sys.argv[2:4]))
