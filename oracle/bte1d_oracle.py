"""CPU oracle of the 1D3V spectral step — TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the reference's spectral 1D3V path (ut-padas/boltzmann,
`BESolver/python/bte_1d3v_solver.py`), used only by `tests/` as the checker. It is pinned to
golden vectors produced by running the reference itself (`tests/golden/make_golden_1d3v.py`).
The velocity-space operators come from `oracle.bte_oracle.Operators` (itself pinned to the
reference's 0D3V goldens); this module adds the 1D3V pieces:

* Chebyshev-Gauss-Lobatto points and collocation derivative (collocation_op.py:8-33);
* ordinates in v-theta (spec_spherical.py:1060-1064) and the ordinate <-> harmonic
  projections (spec_spherical.py:997-1008, m = 0 modes);
* the radial x-advection operator adv_x = M_r^-1 vth (tau / L) int v^3 phi_p phi_k
  (bte_1d3v_solver.py:529-564,621-625) and its eigendecomposition;
* step_bte_x with the backward-Euler Chebyshev operators (bte_1d3v_solver.py:780-887,912-982),
  applied through explicit inverses as the reference does;
* step_bte_v (bte_1d3v_solver.py:984-1137) solved exactly per x point (the reference's GMRES
  converges to this solution within its tolerance);
* initial_condition(type=0) (bte_1d3v_solver.py:1217-1286);
* the fully implicit spectral step: the reference has no such solver (its fully implicit
  step asserts the finite-volume v-space, bte_1d3v_solver.py:1891), so it is composed here
  from the reference's operators as its matvec test composes the coupled operator
  (test_bte_1d_matvec.py:19-83), checked matrix-free against the Kronecker assembly, and
  solved directly at small sizes (or by GMRES, the CPU baseline at full size).
"""
from __future__ import annotations

import math

import numpy as np

from . import bte_oracle as O

TORR = 101325.0 / 760.0
NP0 = 8e16


def chebyshev(Np):
    """collocation_op.py:8-33."""
    deg = Np - 1
    xp = -np.cos(np.pi * np.linspace(0, deg, Np) / deg)
    V0 = np.polynomial.chebyshev.chebvander(xp, deg)
    V0inv = np.linalg.solve(V0, np.identity(Np))
    V1 = np.array([np.polynomial.Chebyshev.basis(i).deriv(m=1)(xp) for i in range(Np)]).reshape((-1, Np)).T
    return xp, V1 @ V0inv


def gl_vt(Nvt):
    """spec_spherical.py:1060-1064 (hspace_split, mode "npsp")."""
    gx, gw = np.polynomial.legendre.leggauss(Nvt // 2)
    return (np.append(np.arccos(0.5 * gx - 0.5), np.arccos(0.5 * gx + 0.5)), np.append(0.5 * gw, 0.5 * gw))


def projections(theta, w, l_max):
    """(psh2o, po2sh), spec_spherical.py:997-1008, Y_l^0 = sqrt((2l+1)/4pi) P_l(cos theta)."""
    Vq = np.zeros((l_max + 1, len(theta)))
    for l in range(l_max + 1):
        c = np.zeros(l + 1)
        c[l] = 1.0
        Vq[l] = math.sqrt((2 * l + 1) / (4 * math.pi)) * np.polynomial.legendre.legval(np.cos(theta), c)
    return Vq.T.copy(), Vq @ np.diag(w) * 2 * np.pi


def radial_v3(ops):
    """compute_spatial_advection_op, bte_1d3v_solver.py:529-564 (one element, no DG)."""
    B = ops.basis
    sp = ops.sp_order
    gx, gw = B.gauss_pn((sp + 8) * B.num_intervals)
    t = B.t
    mm = np.zeros((B.num_p, B.num_p))
    for p in range(B.num_p):
        msk = (gx >= t[p]) & (gx <= t[p + sp + 1])
        x, wq = gx[msk], gw[msk]
        bp = B.eval(p, x)
        for k in range(max(0, p - (sp + 3)), min(B.num_p, p + (sp + 3))):
            mm[p, k] = np.dot(x ** 3 * bp * B.eval(k, x), wq)
    return mm


class Oracle1D:
    def __init__(self, lxcat_file, Np, Nr, Nvt, l_max, ev_max, Te, L, freq, Tg, p0):
        self.ops = ops = O.Operators(O.processes_from_lxcat(lxcat_file), ev_max, Te, Nr + 1, l_max, ee=False,
                                     snap=False)
        self.Np, self.Nr, self.Nvt, self.nsh = Np, Nr + 1, Nvt, l_max + 1
        self.L = 0.5 * L
        self.tau = 1.0 / freq
        self.Tg = Tg
        self.n0 = p0 * TORR / (O.KB * Tg) / NP0
        self.np0 = NP0
        vth = ops.vth
        self.vth = vth
        nsh = self.nsh
        self.op_col_en = ops.op_col_en.sum(axis=0)
        self.op_col_gT = ops.op_col_gT
        self.op_adv_v = ops.op_advection
        Minv_r = ops.Minv[0::nsh, 0::nsh]
        self.op_adv_x = Minv_r @ (vth * (self.tau / self.L) * radial_v3(ops))
        d, Q = np.linalg.eig(self.op_adv_x)
        self.op_adv_x_d, self.op_adv_x_q = d.real, Q.real
        self.op_adv_x_qinv = np.linalg.inv(self.op_adv_x_q)
        self.xp, self.Dp = chebyshev(Np)
        self.xp_vt, self.xp_vt_qw = gl_vt(Nvt)
        self.op_psh2o, self.op_po2sh = projections(self.xp_vt, self.xp_vt_qw, l_max)
        self.Cv = self.tau * self.n0 * self.np0 * (self.op_col_en + Tg * self.op_col_gT)
        self.Av = self.tau * self.op_adv_v

    def ords_to_sph(self, v):
        """bte_1d3v_solver.py:678-685."""
        return np.einsum("li,rix->rlx", self.op_po2sh, v.reshape((self.Nr, self.Nvt, self.Np))).reshape(
            (self.Nr * self.nsh, self.Np))

    def sph_to_ords(self, u):
        """bte_1d3v_solver.py:687-694."""
        return np.einsum("li,rix->rlx", self.op_psh2o, u.reshape((self.Nr, self.nsh, self.Np))).reshape(
            (self.Nr * self.Nvt, self.Np))

    def step_x(self, v, h):
        """step_bte_x with BE Chebyshev operators (bte_1d3v_solver.py:780-887, 912-982)."""
        Nr, Nvt, Np = self.Nr, self.Nvt, self.Np
        DpL = np.zeros((Np, Np))
        DpR = np.zeros((Np, Np))
        DpL[1:, :] = self.Dp[1:, :]
        DpR[:-1, :] = self.Dp[:-1, :]
        Vin = (self.op_adv_x_qinv @ v.reshape((Nr, Nvt * Np))).reshape((Nr * Nvt, Np))
        left = np.array([i * Nvt + j for i in range(Nr) for j in np.where(self.xp_vt <= 0.5 * np.pi)[0]])
        right = np.array([i * Nvt + j for i in range(Nr) for j in np.where(self.xp_vt > 0.5 * np.pi)[0]])
        Vin[left, 0] = 0.0
        Vin[right, -1] = 0.0
        Vin = Vin.reshape((Nr, Nvt, Np))
        out = np.zeros_like(Vin)
        I = np.identity(Np)
        for j in range(Nvt):
            Dj = DpL if self.xp_vt[j] <= 0.5 * np.pi else DpR
            for i in range(Nr):
                Ainv = np.linalg.inv(I + h * self.op_adv_x_d[i] * np.cos(self.xp_vt[j]) * Dj)
                out[i, j] = Ainv @ Vin[i, j]
        return (self.op_adv_x_q @ out.reshape((Nr, Nvt * Np))).reshape((Nr * Nvt, Np))

    def lmat(self, E, u, dt):
        """Lmat_mvec, bte_1d3v_solver.py:1051-1055 (u in (n, Np))."""
        return u - dt * (self.Cv @ u + E[None, :] * (self.Av @ u))

    def step_v(self, E, v, dt):
        """step_bte_v (bte_1d3v_solver.py:984-1137), each point's block solved directly."""
        u = self.ords_to_sph(v)
        n = u.shape[0]
        w = np.zeros_like(u)
        I = np.identity(n)
        for x in range(self.Np):
            w[:, x] = np.linalg.solve(I - dt * (self.Cv + E[x] * self.Av), u[:, x])
        return self.sph_to_ords(w)

    # ---- fully implicit spectral step (composed from the reference's operators) -------------
    def inflow_rows(self):
        """Ordinate indices whose inflow boundary is x = -1 (cos(theta) >= 0) and x = +1 (the
        others), bte_1d3v_solver.py:376-377,936-937."""
        left = np.where(self.xp_vt <= 0.5 * np.pi)[0]
        right = np.where(self.xp_vt > 0.5 * np.pi)[0]
        return left, right

    def _upwinded_d(self):
        """D_L (row 0 zeroed) and D_R (row Np - 1 zeroed), bte_1d3v_solver.py:792-800."""
        Np = self.Np
        DpL = np.zeros((Np, Np))
        DpR = np.zeros((Np, Np))
        DpL[1:, :] = self.Dp[1:, :]
        DpR[:-1, :] = self.Dp[:-1, :]
        return DpL, DpR

    def rhs_vx(self, E, v):
        """The coupled operator of the fully implicit spectral step on ordinates v
        (Nr * Nvt, Np), composed as the reference's matvec test composes it
        (test_bte_1d_matvec.py:19-28): Po (Cv + E_x Av) Ps v - Ax v D^T, with the v-space
        operators of Lmat_mvec (bte_1d3v_solver.py:1051-1055), Ax = adv_x (x) diag(cos theta_j)
        and the upwinded Chebyshev derivative of step_bte_x's set-up (D_L where cos theta_j >= 0,
        D_R otherwise, bte_1d3v_solver.py:792-800,832-839); rows on the inflow boundary are 0."""
        Nr, Nvt, Np = self.Nr, self.Nvt, self.Np
        u = self.ords_to_sph(v)
        yv = self.sph_to_ords(self.Cv @ u + E[None, :] * (self.Av @ u)).reshape((Nr, Nvt, Np))
        DpL, DpR = self._upwinded_d()
        V = v.reshape((Nr, Nvt, Np))
        left, right = self.inflow_rows()
        T = np.zeros_like(V)
        T[:, left] = V[:, left] @ DpL.T
        T[:, right] = V[:, right] @ DpR.T
        yx = np.einsum("rs,j,sjx->rjx", self.op_adv_x, np.cos(self.xp_vt), T)
        y = yv - yx
        y[:, left, 0] = 0.0
        y[:, right, -1] = 0.0
        return y.reshape((Nr * Nvt, Np))

    def fim_operator(self, E, dt):
        """The backward-Euler matrix I - dt L of the fully implicit step, assembled with
        Kronecker products as test_bte_1d_matvec.py:48-83 assembles L (rows of the flattened
        (r, theta, x) state; inflow rows are identity rows). Returns (matrix, inflow rows)."""
        Nr, Nvt, Np = self.Nr, self.Nvt, self.Np
        Ps = np.kron(np.identity(Nr), self.op_po2sh)          # ordinates -> harmonics
        Po = np.kron(np.identity(Nr), self.op_psh2o)          # harmonics -> ordinates
        Cop_o, Av_o = Po @ self.Cv @ Ps, Po @ self.Av @ Ps
        Lv = np.kron(Cop_o, np.identity(Np)) + np.kron(Av_o, np.diag(E))
        DpL, DpR = self._upwinded_d()
        left, right = self.inflow_rows()
        cos = np.cos(self.xp_vt)
        Lx = np.zeros((Nr * Nvt * Np, Nr * Nvt * Np))
        for j in range(Nvt):
            Dj = DpL if j in left else DpR
            Sj = np.zeros((Nvt, Nvt))
            Sj[j, j] = cos[j]
            Lx -= np.kron(np.kron(self.op_adv_x, Sj), Dj)
        L = Lv + Lx
        rows = [(r * Nvt + j) * Np + 0 for r in range(Nr) for j in left]
        rows += [(r * Nvt + j) * Np + Np - 1 for r in range(Nr) for j in right]
        L[rows, :] = 0.0
        return np.identity(L.shape[0]) - dt * L, np.array(rows)

    def step_fim(self, E, v, dt):
        """One fully implicit step: (I - dt L) v_new = v with the inflow values set to 0 (the
        boundary condition step_bte_x imposes, bte_1d3v_solver.py:936-937), solved directly."""
        A, rows = self.fim_operator(E, dt)
        b = np.array(v, dtype=np.float64).reshape(-1).copy()
        b[rows] = 0.0
        return np.linalg.solve(A, b).reshape((self.Nr * self.Nvt, self.Np))

    def step_fim_gmres(self, E, v, dt, rtol=1e-10, restart=30, maxiter=600):
        """The same fully implicit step solved matrix-free, as the reference solves its implicit
        systems (restarted GMRES, utils.py:1172-1262, here SciPy's), right-preconditioned by the
        Lie split the GPU step uses: the exact per-point v-space inverse in FP64, then the
        backward-Euler x-advection over dt. Returns (v_new, iterations); the CPU baseline of
        the fully implicit 1D3V workload."""
        import scipy.sparse.linalg as sla
        Nr, Nvt, Np = self.Nr, self.Nvt, self.Np
        N = Nr * Nvt * Np
        left, right = self.inflow_rows()
        b = np.array(v, dtype=np.float64).reshape((Nr, Nvt, Np)).copy()
        b[:, left, 0] = 0.0
        b[:, right, -1] = 0.0
        n = Nr * self.nsh
        I = np.identity(n)
        blocks = [np.linalg.inv(I - dt * (self.Cv + E[x] * self.Av)) for x in range(Np)]

        def pc(r):
            r = r.reshape((Nr * Nvt, Np))
            u = self.ords_to_sph(r)
            z = np.stack([blocks[x] @ u[:, x] for x in range(Np)], axis=1)
            y = r + self.sph_to_ords(z - u)
            return self.step_x(y, dt).reshape(-1)

        def mv(x):
            x = x.reshape((Nr * Nvt, Np))
            return (x - dt * self.rhs_vx(E, x)).reshape(-1)

        AP = sla.LinearOperator((N, N), matvec=lambda z: mv(pc(z)))
        its = [0]

        def count(_):
            its[0] += 1
        z, info = sla.gmres(AP, b.reshape(-1), rtol=rtol, restart=restart, maxiter=maxiter, callback=count,
                            callback_type="pr_norm")
        return pc(z).reshape((Nr * Nvt, Np)), its[0]

    def step(self, E, v, dt):
        """Strang split, bte_1d3v_solver.py:1885-1889."""
        v = self.step_x(v, 0.5 * dt)
        v = self.step_v(E, v, dt)
        return self.step_x(v, 0.5 * dt)

    def initial_condition(self):
        """initial_condition(type=0) with maxwellian_eedf at the normalisation temperature
        (bte_1d3v_solver.py:1217-1286)."""
        ops, nsh = self.ops, self.nsh
        xx = self.L * (self.xp + 1)
        ne = 1e6 * (1e7 + 1e9 * (1 - 0.5 * xx / self.L) ** 2 * (0.5 * xx / self.L) ** 2) / self.np0
        h = O.maxwellian_initial(ops, 1)[:, 0].copy()
        h[np.arange(len(h)) % nsh != 0] = 0.0
        h = h / np.dot(ops.op_mass, h)
        v = np.einsum("il,rl->ri", self.op_psh2o, h.reshape((self.Nr, nsh))).reshape(-1)
        return np.outer(v, ne)
