"""GB300 1D3V Boltzmann step: spectral v-space (B-splines x spherical harmonics), discrete
ordinates in v-theta, Chebyshev collocation in x.

Counterpart of the spectral path of the reference's `bte_1d3v`
(`BESolver/python/bte_1d3v_solver.py:218-2244`) with its Strang split
(`step`, :1885-1889): x-advection over dt/2 (`step_bte_x`, :912-982), the v-space step over dt
(`step_bte_v`, :984-1137), x-advection over dt/2. The time-step work runs in the CUDA library
(`include/bte1d_gb300.h`); this class builds the setup operators:

* the v-space operators come from the library's own device assembly of the grid (the same
  operators `bte_0d3v_batched` uses): Cv = tau n0 np0 M^-1 (C_en + Tg C_gT), Av = tau M^-1 A;
* the radial x-advection operator adv_x = M_r^-1 vth (tau / L) int v^3 phi_p phi_k and its
  eigendecomposition (:621-625), the ordinate rule (`gl_vt`, spec_spherical.py:1020-1064), the
  ordinate <-> harmonic projections (:997-1008) and the Chebyshev derivative
  (collocation_op.py:8-33) are small dense set-up matrices built on the host.

Differences from the reference, by design: the v-step's GMRES is preconditioned with each
point's own block (I - dt (Cv + E_x Av))^-1 factored in FP32, where the reference uses the
inverse of the nearest of `num_pc_ops` E values (the parameter is read and ignored: the E-binned
inverses are not built, :1333-1344, :889-910, and the exact blocks take their place; GMRES then
converges in a few iterations instead of hundreds, to the same solution within the solver
tolerance). With `solver_type = "fully_implicit"` the step is one backward-Euler step of the
coupled v-space and x-advection operator (`step_fim`), which the reference provides only for
the finite-volume v-space (:1891). Only the BE Chebyshev x-space and the spectral v-space
(the reference's `xspace_type = 1`, `vspace_type = 1`) are provided.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import types

import numpy as np

from . import _lib

QE = 1.602176634e-19
ME = 9.1093837139e-31
KB = 1.380649e-23
TORR = 101325.0 / 760.0
NP0 = 8e16                    # nominal electron density (bte_1d3v_solver.py:103)


def ordinates(Nvt):
    """gl_vt(Nvt, hspace_split=True, mode="npsp") (spec_spherical.py:1060-1064): a Gauss-Legendre
    rule of Nvt/2 points on each half of cos(theta) in [-1, 0] and [0, 1]."""
    gx, gw = np.polynomial.legendre.leggauss(Nvt // 2)
    mu = np.append(0.5 * gx - 0.5, 0.5 * gx + 0.5)
    return np.arccos(mu), np.append(0.5 * gw, 0.5 * gw)


def real_sph_m0(l, theta):
    """Real spherical harmonic Y_l^0(theta): sqrt((2l + 1) / 4 pi) P_l(cos theta)."""
    c = np.zeros(l + 1)
    c[l] = 1.0
    return np.sqrt((2 * l + 1) / (4 * np.pi)) * np.polynomial.legendre.legval(np.cos(theta), c)


def sph_ords_projections(theta, w, l_max):
    """(psh2o [Nvt x nsh], po2sh [nsh x Nvt]) of spec_spherical.py:997-1008 for m = 0 modes."""
    Vq = np.array([real_sph_m0(l, theta) for l in range(l_max + 1)])
    return Vq.T.copy(), (Vq * w[None, :] * 2 * np.pi)


def chebyshev(Np):
    """Chebyshev-Gauss-Lobatto points -cos(pi i / (Np - 1)) and the collocation derivative
    (collocation_op.py:8-33: derivative Vandermonde times the inverse value Vandermonde)."""
    deg = Np - 1
    xp = -np.cos(np.pi * np.linspace(0, deg, Np) / deg)
    V0 = np.polynomial.chebyshev.chebvander(xp, deg)
    V0inv = np.linalg.solve(V0, np.identity(Np))
    V1 = np.array([np.polynomial.Chebyshev.basis(i).deriv(m=1)(xp) for i in range(Np)]).reshape((-1, Np)).T
    return xp, V1 @ V0inv


def load_params(par, fvm=False):
    """The reference's [bte] parameter table (bte_1d3v_solver.py:77-216) from a TOML file path or
    a dict; returns a namespace with the derived quantities the step uses. `fvm`: the table is
    for the finite-volume v-space (`vspace_type = 0`), with either x-space."""
    if isinstance(par, (str, os.PathLike)):
        import tomllib
        with open(par, "rb") as fh:
            tp = tomllib.load(fh)["bte"]
    else:
        tp = dict(par)
    p = types.SimpleNamespace(**tp)
    p.L = 0.5 * tp["L"]
    p.f = tp["freq"]
    p.tau = 1.0 / p.f
    p.Tg = tp["Tg"]
    p.p0 = tp["p0"]
    n0 = p.p0 * TORR / (KB * p.Tg) if p.Tg != 0 else 3.22e22 * p.p0
    p.np0 = NP0
    p.n0 = n0 / NP0
    p.l_max = tp["lmax"]
    p.gmres_rsrt_iter = tp.get("gmres_rsrt_iter", 10)
    p.gmres_maxiter = p.gmres_rsrt_iter * tp["gmres_rsrt"]
    if fvm:
        if tp.get("vspace_type", 1) != 0:
            raise ValueError("the finite-volume solver needs vspace_type = 0")
        if tp.get("xspace_type", 1) not in (0, 1):
            raise NotImplementedError("xspace_type must be 0 (upwind FD) or 1 (Chebyshev)")
    elif tp.get("xspace_type", 1) != 1 or tp.get("vspace_type", 1) != 1:
        raise NotImplementedError("only the BE Chebyshev x-space and the spectral v-space are provided")
    if tp.get("ev_extend", 0) != 0:
        raise NotImplementedError("only ev_extend = 0 (the v-grid ends at ev_max)")
    return p


def write_checkpoint(fprefix, v, time, dt, ne, Te):
    """store_checkpoint (bte_1d3v_solver.py:2065-2090) in NumPy's .npz format (the reference
    writes HDF5, whose library this package does not use): `fprefix`.npz with the reference's
    dataset names "time[T]", "dt[T]", "edf", "ne[m^-3]" and "Te[eV]". Raises OSError on a
    failed write (the reference prints and carries on)."""
    host = lambda a: a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
    with open("%s.npz" % fprefix, "wb") as fh:
        np.savez(fh, **{"time[T]": np.array([float(time)]), "dt[T]": np.array([float(dt)]), "edf": host(v),
                        "ne[m^-3]": host(ne), "Te[eV]": host(Te)})


def read_checkpoint(fprefix):
    """restore_checkpoint (bte_1d3v_solver.py:2092-2103): (time, dt, edf) from `fprefix`.npz."""
    with np.load("%s.npz" % fprefix) as F:
        return float(F["time[T]"][0]), float(F["dt[T]"][0]), np.array(F["edf"])


def spectral_qoi_rows(mass, temp, rates, vth, nsh):
    """The spectral grid's QoI rows (bte_1d3v_solver.py:588-598) over the n = Nr * nsh
    coefficients: mass (utils.mass_op), temperature in eV (utils.temp_op vth^2 0.5 me (2/3/kB) /
    (e/kB): `temp` is the grid's TEMP_VEC export, without the vth^2), and per process the rate
    functional (n_proc x Nr) on the l = 0 coefficients. Returns (2 + n_proc) x n."""
    mass, temp, rates = (np.asarray(a, dtype=np.float64) for a in (mass, temp, rates))
    Q = np.zeros((2 + rates.shape[0], mass.shape[0]))
    Q[0], Q[1] = mass, temp * vth ** 2
    Q[2:, 0::nsh] = rates
    return Q


class bte_1d3v:
    """Spectral 1D3V solver on one GPU. `par` is the reference's parameter file (TOML with a
    [bte] table) or the same table as a dict; `collisions` in it names an LXCat file."""

    def __init__(self, par, device=0):
        import torch
        from .bte_0d3v_batched import bte_0d3v_batched, vspace_grid_extension
        self.torch = torch
        self.params = p = load_params(par)
        self.device = device
        torch.cuda.set_device(device)
        Nr = p.Nr + 1
        nsh = p.l_max + 1
        self.dof_vr, self.dof_vt, self.dof_x = Nr, p.Nvt, p.Np
        self.num_sh = nsh
        self.dof_v = Nr * nsh
        # the velocity grid and its operators, assembled on the device
        args = types.SimpleNamespace(threads=1, sp_order=p.sp_order, spline_qpts=p.spline_qpts, ee_collisions=0,
                                     verbose=0, use_gpu=1, Efreq=0.0, dt=p.dt, cycles=1, solver_type="steady-state",
                                     l_max=p.l_max, Nr=p.Nr, n_pts=p.Np, precision="fp64")
        s = bte_0d3v_batched(args, np.array([float(p.ev_max)]), np.array([float(p.Te)]), np.array([p.Nr]),
                             [[[l, 0] for l in range(nsh)]], 1, [p.collisions])
        s._dev_id = device
        s._plain_knots = 1  # the 1D3V basis has no threshold knots (bte_1d3v_solver.py:356, sig_pts=None)
        s.assemble_operators(0, vspace_ext=vspace_grid_extension.NONE)
        self.grid = s
        info = s._grid_info[0]
        self.vth = info["vth"]
        n = info["n"]
        Minv = s.export_operator(0, "MINV")
        col = s.export_operator(0, "COL_RAW").sum(dim=0)
        colT = s.export_operator(0, "COL_GT_RAW")
        adv = s.export_operator(0, "ADV_RAW") * ((1.0 / self.vth) * (QE / ME))
        self.op_col_en = Minv @ col
        self.op_col_gT = Minv @ colT
        self.op_adv_v = Minv @ adv
        Cv = p.tau * p.n0 * p.np0 * (self.op_col_en + p.Tg * self.op_col_gT)
        Av = p.tau * self.op_adv_v
        # radial x-advection operator and its eigendecomposition (bte_1d3v_solver.py:529-564,621-625)
        Mr_inv = Minv[0::nsh, 0::nsh]
        v3 = torch.empty((Nr, Nr), dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().bte_grid_export(s._grid[0], _lib.OP["RADIAL_V3"], _lib.ptr(v3), v3.numel(),
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream)), "bte_grid_export")
        adv_x = (Mr_inv @ (self.vth * (p.tau / p.L) * v3)).cpu().numpy()
        d, Q = np.linalg.eig(adv_x)
        if np.max(np.abs(d.imag)) > 1e-12 * np.max(np.abs(d.real)):
            raise RuntimeError("the radial x-advection operator has complex eigenvalues")
        d, Q = d.real.copy(), Q.real.copy()
        Qinv = np.linalg.inv(Q)
        self.op_adv_x, self.op_adv_x_d, self.op_adv_x_q, self.op_adv_x_qinv = adv_x, d, Q, Qinv
        self.xp_vt, self.xp_vt_qw = ordinates(p.Nvt)
        self.op_psh2o, self.op_po2sh = sph_ords_projections(self.xp_vt, self.xp_vt_qw, p.l_max)
        self.xp, self.Dp = chebyshev(p.Np)
        lib = _lib.load()
        dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in
                      (Q, Qinv, d, np.cos(self.xp_vt), self.Dp, self.op_po2sh, self.op_psh2o,
                       Cv.cpu().numpy(), Av.cpu().numpy())]
        h = C.c_void_p()
        rc = lib.bte1d_create(int(device), Nr, nsh, int(p.Nvt), int(p.Np), *[dp(a) for a in self._keep],
                              int(p.gmres_rsrt), C.byref(h))
        if rc != 0:
            raise RuntimeError("bte1d_create failed (%d): %s" % (rc, lib.bte1d_last_error().decode()))
        self._h = h
        self.mass_op = s.export_operator(0, "MASS_VEC")
        st = str(getattr(p, "solver_type", "strang")).lower()
        if st in ("2", "fully_implicit"):
            self.solver = "fully_implicit"
        elif st in ("0", "strang", "xvx_strang_split", "none"):
            self.solver = "strang"
        else:
            raise NotImplementedError("solver_type must be the Strang split or fully_implicit for the spectral v-space")
        self.op_qoi = None   # the QoI rows, built on the first compute_qoi
        self.gmres_info = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.load().bte1d_destroy(h)
            self._h = None

    # ------------------------------------------------------------------ helpers
    def _s(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed (%d): %s" % (what, rc, _lib.load().bte1d_last_error().decode()))

    def _dev(self, a, shape):
        t = self.torch.as_tensor(a, dtype=self.torch.float64, device="cuda")
        return t.reshape(shape).contiguous()

    # ------------------------------------------------------------------ reference interface
    def init(self, dt):
        """The reference's init(dt) (:1333-1344) builds num_pc_ops E-binned preconditioner
        inverses; here each point's exact block is factored inside each v-step instead
        (num_pc_ops is ignored), so only dt is recorded."""
        self.params.dt = dt

    def ords_to_sph(self, x):
        """(Nr * Nvt, Nx) ordinates -> (Nr * nsh, Nx) harmonic coefficients (:678-685)."""
        V = self._dev(x, (self.dof_vr * self.dof_vt, self.dof_x))
        U = self.torch.empty((self.dof_x, self.dof_v), dtype=self.torch.float64, device="cuda")
        self._check(_lib.load().bte1d_ords_to_lm(self._h, _lib.ptr(V), _lib.ptr(U), self._s()), "bte1d_ords_to_lm")
        return U.t().contiguous()

    def sph_to_ords(self, x):
        """(Nr * nsh, Nx) harmonic coefficients -> (Nr * Nvt, Nx) ordinates (:687-694)."""
        U = self._dev(x, (self.dof_v, self.dof_x)).t().contiguous()
        V = self.torch.empty((self.dof_vr * self.dof_vt, self.dof_x), dtype=self.torch.float64, device="cuda")
        self._check(_lib.load().bte1d_lm_to_ords(self._h, _lib.ptr(U), _lib.ptr(V), self._s()), "bte1d_lm_to_ords")
        return V

    def lmat_mvec(self, E, x, dt):
        """Lmat_mvec of step_bte_v (:1051-1055): x - dt tau (n0 np0 (C + Tg C_T) x + E A x), x (n, Nx)."""
        X = self._dev(x, (self.dof_v, self.dof_x)).t().contiguous()
        Ed = self._dev(E, (self.dof_x,))
        Y = self.torch.empty_like(X)
        self._check(_lib.load().bte1d_lmat(self._h, float(dt), _lib.ptr(Ed), _lib.ptr(X), _lib.ptr(Y), self._s()),
                    "bte1d_lmat")
        return Y.t().contiguous()

    def block_solve(self, E, x, dt):
        """Per-point block inverse (I - dt (Cv + E_x Av))^-1 x in FP32 (the v-step's preconditioner), x (n, Nx)."""
        X = self._dev(x, (self.dof_v, self.dof_x)).t().contiguous()
        Ed = self._dev(E, (self.dof_x,))
        Y = self.torch.empty_like(X)
        self._check(_lib.load().bte1d_block_solve(self._h, float(dt), _lib.ptr(Ed), _lib.ptr(X), _lib.ptr(Y),
                                                  self._s()), "bte1d_block_solve")
        return Y.t().contiguous()

    def step_bte_x(self, v, time, dt, verbose=0):
        """Backward-Euler x-advection over dt (:912-982); returns the new (Nr * Nvt, Nx) state."""
        V = self._dev(v, (self.dof_vr * self.dof_vt, self.dof_x)).clone()
        self._check(_lib.load().bte1d_step_x(self._h, float(dt), _lib.ptr(V), self._s()), "bte1d_step_x")
        return V

    def step_bte_v(self, E, v, dv, time, dt, verbose=0, atol=None, rtol=None, max_iter=None):
        """v-space step over dt at field E (:984-1137); returns the new ordinates state."""
        p = self.params
        V = self._dev(v, (self.dof_vr * self.dof_vt, self.dof_x)).clone()
        Ed = self._dev(E, (self.dof_x,))
        info = (C.c_double * 4)()
        rc = _lib.load().bte1d_step_v(self._h, float(dt), _lib.ptr(Ed), _lib.ptr(V),
                                       float(p.rtol if rtol is None else rtol), float(p.atol if atol is None else atol),
                                       int(p.gmres_maxiter if max_iter is None else max_iter), info, self._s())
        self._check(rc, "bte1d_step_v")
        self.gmres_info = {"iterations": int(info[0]), "residual_abs": info[1], "residual_rel": info[2],
                           "status": int(info[3])}
        if info[3] != 0:
            raise RuntimeError("GMRES did not converge: iterations=%d ||res||/||b||=%.4e" % (info[0], info[2]))
        return V

    def step(self, E, v, dv, time, dt, verbose=0):
        """One step of the configured solver: the Strang split (:1885-1889: x over dt/2, v over
        dt, x over dt/2), or with solver_type "fully_implicit" one backward-Euler step of the
        coupled v-space and x-advection operator (step_fim)."""
        if self.solver == "fully_implicit":
            return self.step_fim(E, v, time, dt)
        v = self.step_bte_x(v, time, 0.5 * dt)
        v = self.step_bte_v(E, v, None, time, dt)
        return self.step_bte_x(v, time + 0.5 * dt, 0.5 * dt)

    def fim_mvec(self, E, v, dt):
        """The fully implicit step's operator on ordinates v (Nr * Nvt, Nx):
        v - dt (P_sh2o (Cv + E_x Av) P_o2sh v - (adv_x (x) cos theta) v D^T), identity rows on the
        inflow boundary. The reference's fully implicit solver takes only the finite-volume
        v-space (:1891); this operator composes its spectral operators (Lmat_mvec, :1051-1055,
        and step_bte_x's BE Chebyshev advection, :912-982) as its matvec test composes them
        (test_bte_1d_matvec.py:19-83)."""
        V = self._dev(v, (self.dof_vr * self.dof_vt, self.dof_x))
        Ed = self._dev(E, (self.dof_x,))
        Y = self.torch.empty_like(V)
        self._check(_lib.load().bte1d_fim_matvec(self._h, float(dt), _lib.ptr(Ed), _lib.ptr(V), _lib.ptr(Y),
                                                 self._s()), "bte1d_fim_matvec")
        return Y

    def step_fim(self, E, v, time, dt, atol=None, rtol=None, max_iter=None, pc=None):
        """One fully implicit step over dt at field E: fim_mvec(v_new) = v (inflow values 0) by
        right-preconditioned GMRES(gmres_rsrt) to rtol (params rtol, 1e-10 in the 1D3V tables);
        the preconditioner is a Lie split, the per-point v-space block inverse (FP32 factors)
        then the backward-Euler x-advection over dt (pc "split", default), or the v blocks alone
        (pc "vblock"). gmres_info holds the iterations and residuals."""
        p = self.params
        pc = getattr(p, "fim_pc", "split") if pc is None else pc
        if pc not in ("split", "vblock"):
            raise ValueError("pc must be 'split' or 'vblock'")
        V = self._dev(v, (self.dof_vr * self.dof_vt, self.dof_x)).clone()
        Ed = self._dev(E, (self.dof_x,))
        info = (C.c_double * 4)()
        rc = _lib.load().bte1d_step_fim(self._h, float(dt), _lib.ptr(Ed), _lib.ptr(V),
                                         float(p.rtol if rtol is None else rtol), float(p.atol if atol is None else atol),
                                         int(p.gmres_maxiter if max_iter is None else max_iter),
                                         0 if pc == "split" else 1, info, self._s())
        self._check(rc, "bte1d_step_fim")
        self.gmres_info = {"iterations": int(info[0]), "residual_abs": info[1], "residual_rel": info[2],
                           "status": int(info[3])}
        if info[3] != 0:
            raise RuntimeError("GMRES did not converge: iterations=%d ||res||/||b||=%.4e" % (info[0], info[2]))
        return V

    def initial_condition(self, type=0):
        """initial_condition(type=0) (:1274-1286, maxwellian_eedf :1217-1272): a Maxwellian at the
        normalisation temperature at every point, mass-normalized, times the density profile."""
        if type != 0:
            raise NotImplementedError
        p = self.params
        xx = p.L * (self.xp + 1)
        ne = 1e6 * (1e7 + 1e9 * (1 - 0.5 * xx / p.L) ** 2 * (0.5 * xx / p.L) ** 2) / p.np0
        f0 = self.torch.as_tensor(self.grid.initialize(0, 1)[:, 0], device="cuda")
        h = f0 / (self.mass_op @ f0)
        vo = (self.torch.as_tensor(self.op_psh2o, device="cuda") @ h.reshape(self.dof_vr, self.num_sh).t()).t()
        return vo.reshape(-1, 1) * self.torch.as_tensor(ne, device="cuda")[None, :]

    def compute_qoi(self, v, time, dt):
        """compute_qoi (:1179-1215) per x point from the ordinates v: "rates" (Nx, n_proc), "ne",
        "Te"; "mu" and "D" are 0 as in the reference. The harmonics of v meet the QoI rows in
        one FP64 GEMM (bte_dgemm_nn)."""
        from .bte_1d3v_fvm import qoi_from_moments
        if self.op_qoi is None:
            s = self.grid
            rows = spectral_qoi_rows(self.mass_op.cpu().numpy(), s.export_operator(0, "TEMP_VEC").cpu().numpy(),
                                     s.export_operator(0, "RATES").cpu().numpy(), self.vth, self.num_sh)
            self.op_qoi = self.torch.as_tensor(rows, dtype=self.torch.float64, device="cuda")
        U = self.ords_to_sph(v).contiguous()
        Q = self.op_qoi
        Y = self.torch.empty((Q.shape[0], self.dof_x), dtype=self.torch.float64, device="cuda")
        rc = _lib.load().bte_dgemm_nn(Q.shape[0], self.dof_x, self.dof_v, _lib.ptr(Q), self.dof_v, _lib.ptr(U),
                                      self.dof_x, _lib.ptr(Y), self.dof_x, self._s())
        if rc != 0:
            raise RuntimeError("QoI functionals failed (%d): %s" % (rc, _lib.load().bte_sweep_last_error().decode()))
        return qoi_from_moments(Y, self.vth, self.params.np0, math.sqrt(4.0 * math.pi))

    def store_checkpoint(self, v, time, dt, fprefix):
        """store_checkpoint (:2065-2090): v with its ne and Te, to `fprefix`.npz."""
        q = self.compute_qoi(v, time, dt)
        write_checkpoint(fprefix, v, time, dt, q["ne"], q["Te"])

    def restore_checkpoint(self, fprefix):
        """restore_checkpoint (:2092-2103): (time, dt, v) with v on the device."""
        t, dt, v = read_checkpoint(fprefix)
        return t, dt, self.torch.as_tensor(v, dtype=self.torch.float64, device="cuda")

    def normalize_edf(self, v):
        """normalize_edf (:2043-2055): the ordinates v divided, per x, by the mass functional of
        their harmonics in the reference's units, (mass . v_lm) / sqrt(4 pi) 2 (vth / c_gamma)^3."""
        from .bte_0d3v_batched import normalization_scale
        V = self.torch.as_tensor(v, dtype=self.torch.float64, device="cuda").reshape(self.dof_vr * self.dof_vt,
                                                                                      self.dof_x)
        return V / normalization_scale(self.mass_op, self.ords_to_sph(V), self.vth)

    def asnumpy(self, x):
        return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)

    def copy_operators_H2D(self, dev_id=0):
        """The operators live on the device from construction on: nothing to copy."""

    def copy_operators_D2H(self, dev_id=0):
        """The operators stay on the device; their host copies are the set-up matrices."""

    def compute_radial_components(self, ev, v):
        """compute_radial_components (:1139-1160): f_l(eps) of the ordinates v at the energies ev
        (eV), (Nx, num_sh, len(ev)) NumPy array, from the grid's B-spline evaluation
        (bte_radial_components) on the harmonics of v."""
        return self.grid.compute_radial_components(0, ev, self.ords_to_sph(v))

    def launches(self):
        return int(_lib.load().bte1d_launches(self._h))
