"""CPU oracle of the finite-volume 1D3V op-split step — TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the reference's `bte_1d3v.step_op_split` with type XVTVRC
(ut-padas/boltzmann, `BESolver/python/bte_1d3v_solver.py:1745-1870`). Layout of v: (Nr * Nvt, Nx),
radial cell r major, ordinate j minor. The step:

1. collisions: yc = PmatC v, PmatC the inverse of I - dt tau n0 np0 (C_en + Tg C_gT) on the FVM
   v-grid (:1346-1375, dense at small sizes);
2. v_r advection: lines (x, j) of Nr cells, upwind backward Euler with a = -aE[x] cos(theta_j),
   aE = tau qe / (me vth) E (:1775, :1803-1808);
3. v_theta advection: lines (x, r) of Nvt cells, a = aE[x] / v_r (:1822-1826);
4. x advection: inflow values zeroed (theta <= pi/2 at the first x point, > pi/2 at the last),
   lines (r, j) of Nx cells, a = vth (tau / L) v_r cos(theta_j) (:1776, :1834-1853).

The sweeps are `oracle.sweeps_oracle` (pinned to dense solves); `tests/golden/make_golden_fvm.py`
pins this composition to the reference's own step.
"""
from __future__ import annotations

import numpy as np

from . import sweeps_oracle as SO


def op_split_step(g, E, v, dt, alpha=1.0):
    """g: the fixture's set-up (dict-like: Nr, Nvt, Nx, pvr, pvt, px, tau, qe, me, vth, L, vr,
    vt, PmatC and the six column-stored band arrays). Returns the new v (Nr * Nvt, Nx)."""
    Nr, Nvt, Nx = int(g["Nr"]), int(g["Nvt"]), int(g["Nx"])
    aE = (float(g["tau"]) * float(g["qe"]) / float(g["me"]) / float(g["vth"])) * np.asarray(E)
    ax = float(g["vth"]) * (float(g["tau"]) / float(g["L"]))
    vr, vt = np.asarray(g["vr"]), np.asarray(g["vt"])
    cos_vt = np.cos(vt)
    h = alpha * dt
    yc = np.asarray(g["PmatC"]) @ v.reshape(Nr * Nvt, Nx)
    y = np.swapaxes(yc.reshape(Nr, Nvt, Nx), 0, 2)                          # (Nx, Nvt, Nr)
    nd = int(g["pvr"]) + 1
    y = SO.adv_vr_BE(g["vr_diag_l2r"][:nd], g["vr_diag_r2l"][:nd], aE, cos_vt, h, y.reshape(-1), Nr, Nvt, Nx)
    y = np.swapaxes(y.reshape(Nx, Nvt, Nr), 1, 2)                           # (Nx, Nr, Nvt)
    nd = int(g["pvt"]) + 1
    y = SO.adv_vt_BE(g["vt_diag_l2r"][:nd], g["vt_diag_r2l"][:nd], aE, vr, h, y.reshape(-1), Nr, Nvt, Nx)
    y = np.swapaxes(np.swapaxes(y.reshape(Nx, Nr, Nvt), 0, 2), 0, 1).copy()  # (Nr, Nvt, Nx)
    y[:, vt <= 0.5 * np.pi, 0] = 0.0
    y[:, vt > 0.5 * np.pi, -1] = 0.0
    nd = int(g["px"]) + 1
    y = SO.adv_x_BE(g["x_diag_l2r"][:nd], g["x_diag_r2l"][:nd], ax * vr, cos_vt, h, y.reshape(-1), Nr, Nvt, Nx)
    return y.reshape(Nr * Nvt, Nx)
