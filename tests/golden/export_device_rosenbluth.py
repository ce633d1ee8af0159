"""Export the library's assembled Rosenbluth-potential operators (HL, GL) of the c2-shape grid
(128 B-splines, l_max 2) to an .npz file, for make_golden_c2.py --swap-rosenbluth.

Runs on a GPU host with the library built. The swap experiment rebuilds the reference's Coulomb
operator from the reference's own trilinear tensors and these device potentials, and solves
again with the reference, to separate how much of the difference between the device solution
and the reference's comes from the potentials alone.

Usage:  python tests/golden/export_device_rosenbluth.py OUT.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..")))

from helpers import gpu_solver  # noqa: E402
from boltzmann_gb300.workloads import write_synthetic_lxcat  # noqa: E402


def main(out):
    xs = write_synthetic_lxcat()
    try:
        s, _ = gpu_solver(xs, 128, 2, True, 1, "fp64")
        np.savez_compressed(out, hl=s.export_operator(0, "HL").cpu().numpy(),
                            gl=s.export_operator(0, "GL").cpu().numpy(),
                            minv=s.export_operator(0, "MINV").cpu().numpy())
    finally:
        os.unlink(xs)


if __name__ == "__main__":
    main(sys.argv[1])
