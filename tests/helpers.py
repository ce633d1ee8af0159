"""Shared test helpers: build the drop-in solver and the CPU oracle on the same inputs."""
import types

import numpy as np

from boltzmann_gb300.workloads import EV_MAX, TE_NORM, batch_parameters, config_parameters


def make_args(n_sp, l_max, ee, n_pts, precision="fp64"):
    return types.SimpleNamespace(threads=1, sp_order=3, spline_qpts=5, ee_collisions=int(ee), verbose=0, use_gpu=1,
                                 Efreq=0.0, dt=1e-3, cycles=1, solver_type="steady-state", l_max=l_max, Nr=n_sp - 1,
                                 n_pts=n_pts, precision=precision)


def params_for(ee, n_pts, seed=20261203):
    if ee:
        return batch_parameters(n_pts, seed)
    p = config_parameters("c1", n_pts)
    return p


def gpu_solver(xs, n_sp, l_max, ee, n_pts, precision="fp64", ext=0):
    from boltzmann_gb300.bte_0d3v_batched import bte_0d3v_batched, vspace_grid_extension
    args = make_args(n_sp, l_max, ee, n_pts, precision)
    s = bte_0d3v_batched(args, np.array([EV_MAX]), np.array([TE_NORM]), np.array([n_sp - 1]),
                         [[[l, 0] for l in range(l_max + 1)]], 1, [xs])
    s.assemble_operators(0, vspace_ext=vspace_grid_extension(ext))
    return s, args


def oracle_ops(xs, n_sp, l_max, ee, ext=False, dense=True):
    from oracle import bte_oracle as O
    return O.Operators(O.processes_from_lxcat(xs), EV_MAX, TE_NORM, n_sp, l_max, ee=ee, extend_linear=ext,
                       dense_coulomb=dense)


def relmax(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel_l2_cols(a, b):
    """Per-column relative L2 error of (n, P) arrays."""
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)


# the parameter table of the finite-volume fixtures (tests/golden/make_golden_fvm_implicit.py:
# the 1D3V golden table with the FVM v-space, upwind x, stencil orders 2, fully implicit)
FVM_IMPLICIT_PARAMS = dict(L=2.54e-2, V0=100.0, freq=13.56e6, Tg=300.0, p0=1.0, gmres_rsrt=30, gmres_rsrt_iter=20,
                           Np=12, Nr=7, Nvt=8, lmax=1, dt=1e-3, ev_max=80.0, ev_extend=0, sp_order=3, spline_qpts=5,
                           Te=4.0, xspace_type=0, vspace_type=0, solver_type="fully_implicit", adaptive_grid=1, pvr=2,
                           pvt=2, px=2, rtol=1e-12, atol=1e-14, ic_file="")

# the semi-Lagrangian fixture's table (tests/golden/make_golden_fvm_sl.py)
FVM_SL_PARAMS = dict(FVM_IMPLICIT_PARAMS, solver_type="sl_implicit", dt=5e-3)
