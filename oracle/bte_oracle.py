"""CPU oracle for the batched 0D3V velocity-space path — TEST INFRASTRUCTURE ONLY.

This is a NumPy/SciPy restatement of the reference's algorithm (ut-padas/boltzmann,
`BESolver/python/`), used only by `tests/`, `__graft_entry__.smoke()` and the CPU
baseline legs of `bench.py`, always as the checker and never as the product. The CUDA
library in `boltzmann_gb300/csrc` is the product; nothing in `boltzmann_gb300/` imports
this file.

Each function cites the reference code it restates. Vectorisation replaces the
reference's per-(p,k) Python loops and its process pool; the arithmetic (quadrature
rules, masks, constants, operator definitions, Newton / line-search logic) is the
reference's. Parity of this oracle is pinned against golden vectors produced by running
the reference itself (`tests/golden/make_golden.py`).

The one piece not restated literally is the Coulomb integrand table
`cc_terms.Ia/Ib` (sympy output of `sym_cc.assemble_symbolic_cc_op`,
`BESolver/python/sym_cc.py:28-80`): the same weak forms are re-derived in closed
form in `coulomb_angular_tables` (gradient and covariant-Hessian contractions in
(v, mu=cos theta, phi) coordinates, Legendre identity used to remove Y''), with the
mu-integrals done by Gauss-Legendre quadrature, which is exact for these polynomials.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.interpolate
import scipy.linalg

# scipy.constants values (CODATA 2018, as in the reference environment).
QE = 1.602176634e-19
ME = 9.1093837139e-31
KB = 1.380649e-23
EPS0 = 8.8541878188e-12
EV = 1.602176634e-19
QE_BY_ME = QE / ME
TEMP_K_1EV = EV / KB                 # collisions.py:39
C_GAMMA = math.sqrt(2.0 * QE_BY_ME)  # bte_0d3v_batched.py:163


def electron_thermal_velocity(T_kelvin):
    """collisions.py:20-25."""
    return np.sqrt(2.0 * KB * T_kelvin / ME)


# ----------------------------------------------------------------------------------
# B-spline basis (basis.py:327-767)
# ----------------------------------------------------------------------------------
def uniform_knots(k_domain, num_p, sp_order):
    """basis.py:640-653."""
    t = k_domain[0] * np.ones(sp_order)
    t = np.append(t, np.linspace(k_domain[0], k_domain[1], num_p - sp_order, endpoint=False))
    t = np.append(t, k_domain[1] * np.ones(sp_order + 1))
    return t


def snap_knots(t, k_domain, sp_order, sig_pts):
    """Threshold-knot snapping, basis.py:356-362."""
    t = t.copy()
    for s in sig_pts:
        if k_domain[0] < s < k_domain[1]:
            idx = int(np.argmin(np.abs(t - s)))
            if sp_order + 1 < idx < len(t) - sp_order - 1:
                t[idx] = s
    return t


class Basis:
    """Cubic (any order) B-spline basis with the reference's evaluation semantics:
    each basis function is `scipy.interpolate.BSpline.basis_element(t[i:i+k+2],
    extrapolate=False)` with NaN (outside its support) mapped to 0 (basis.py:387,411-412);
    derivatives use the standard recursion (basis.py:460-501)."""

    def __init__(self, t, sp_order):
        self.t = np.asarray(t, dtype=np.float64)
        self.k = sp_order
        self.num_p = len(self.t) - (sp_order + 1)
        self._el = [scipy.interpolate.BSpline.basis_element(self.t[i:i + sp_order + 2], False)
                    for i in range(self.num_p)]
        self._d = {}
        self.t_unique = np.unique(self.t)
        self.num_intervals = len(self.t_unique) - 1

    def eval(self, i, x, d=0):
        if d == 0:
            return np.nan_to_num(self._el[i](x))
        return np.nan_to_num(self.deriv(i, d)(x))

    def deriv(self, i, d):
        """basis.py:460-501: f1 * sum_j f_alpha(d, j) * B_{i+j, k-d}."""
        key = (i, d)
        if key in self._d:
            return self._d[key]
        t, p = self.t, self.k
        f1 = math.factorial(p) / math.factorial(p - d)

        def f_alpha(kk, j):
            if kk == 0 and j == 0:
                return 1.0
            if j == 0:
                d1 = t[i + p - kk + 1] - t[i]
                return f_alpha(kk - 1, 0) / d1 if d1 != 0 else 0.0
            if 0 < j < kk:
                d1 = t[i + p + j - kk + 1] - t[i + j]
                return (f_alpha(kk - 1, j) - f_alpha(kk - 1, j - 1)) / d1 if d1 != 0 else 0.0
            d1 = t[i + p + 1] - t[i + kk]
            return -f_alpha(kk - 1, kk - 1) / d1 if d1 != 0 else 0.0

        parts = []
        for j in range(d + 1):
            el = scipy.interpolate.BSpline.basis_element(t[i + j:(i + j) + (p - d) + 2], False)
            parts.append((f_alpha(d, j), el))

        def fn(x):
            y = 0.0
            for c, el in parts:
                y = y + c * np.nan_to_num(el(x))
            return y * f1

        self._d[key] = fn
        return fn

    def vandermonde(self, x, d=0):
        """(num_p, len(x)) matrix of basis values (or derivatives) at x."""
        return np.array([self.eval(i, x, d) for i in range(self.num_p)])

    def gauss_pn(self, deg):
        """Per-knot-interval Gauss-Legendre rule, basis.py:414-429."""
        q = deg // self.num_intervals
        gx, gw = np.polynomial.legendre.leggauss(q)
        qx, qw = [], []
        t = self.t
        for i in range(len(t) - 1):
            if t[i] != t[i + 1]:
                qx.append(0.5 * (t[i + 1] - t[i]) * gx + 0.5 * (t[i + 1] + t[i]))
                qw.append(0.5 * (t[i + 1] - t[i]) * gw)
        qx, qw = np.concatenate(qx), np.concatenate(qw)
        assert np.allclose(np.sum(qw), t[-1] - t[0], rtol=1e-14, atol=1e-14)
        return qx, qw

    def support_mask(self, i, x):
        return np.logical_and(x >= self.t[i], x <= self.t[i + self.k + 1])


# ----------------------------------------------------------------------------------
# Cross sections (collisions.py:64-79, 235-262)
# ----------------------------------------------------------------------------------
class Process:
    """One electron-heavy process with linear, end-clamped sigma(eps) interpolation."""

    TYPES = {"ELASTIC": 0, "EXCITATION": 1, "IONIZATION": 2, "ATTACHMENT": 3}

    def __init__(self, name, data, mByM):
        self.name = name
        self.kind = data["type"]
        self.gtype = Process.TYPES[self.kind]
        self.energy = np.asarray(data["energy"], dtype=np.float64)
        self.sigma = np.asarray(data["cross section"], dtype=np.float64)
        self.threshold = data["threshold"]
        self.species = data["species"]
        self.mByM = mByM
        self.attachment_energy = 0.0
        if self.kind == "ATTACHMENT":
            self.attachment_energy = float(data["info"].get("FORWARD", 0.0))
        self._interp = scipy.interpolate.interp1d(self.energy, self.sigma, kind="linear",
                                                  bounds_error=False,
                                                  fill_value=(self.sigma[0], self.sigma[-1]))

    def total_cross_section(self, eps):
        return self._interp(eps)


# ----------------------------------------------------------------------------------
# Operators
# ----------------------------------------------------------------------------------
def sph_harm_norm(l):
    """advection_operator_spherical_polys.py:6-10 (m = 0)."""
    return np.sqrt((2.0 * l + 1) / (4.0 * np.pi))


def AM(l):
    return (l) / (2.0 * l + 1.0) * sph_harm_norm(l) / sph_harm_norm(l - 1)


def BM(l):
    return (l + 1.0) / (2.0 * l + 1.0) * sph_harm_norm(l) / sph_harm_norm(l + 1)


def AD(l):
    return (l) * (l + 1.0) / (2.0 * l + 1.0) * sph_harm_norm(l) / sph_harm_norm(l - 1)


def BD(l):
    return -l * (l + 1.0) / (2.0 * l + 1.0) * sph_harm_norm(l) / sph_harm_norm(l + 1)


def _place_blocks(blocks_by_l, lm, num_p):
    """Scatter per-l radial blocks into the radial-major (p*num_sh + lm) layout."""
    num_sh = len(lm)
    out = np.zeros((num_p * num_sh, num_p * num_sh))
    for li, (l, _) in enumerate(lm):
        b = blocks_by_l(l)
        if b is not None:
            out[li::num_sh, li::num_sh] = b
    return out


def coulomb_angular_tables(l_max, nq=None):
    """Angular coefficients of the Coulomb weak forms for every (q, l, s) triple.

    Restates the weak forms of `sym_cc.assemble_symbolic_cc_op` (sym_cc.py:28-56):
        Ia = 2 pi v^2 * int (grad psi . grad h) f dmu
        Ib =   pi v^2 * int (Hess psi : Hess g) f dmu
    with psi = B_p Y_q, f = B_k Y_l, h, g = B_r Y_s, Y_l = sqrt((2l+1)/4pi) P_l(mu),
    metric diag(1, v^2/(1-mu^2), v^2 (1-mu^2)). With a = 1 - mu^2 and
    Z_l = mu Y_l' - l(l+1) Y_l (the Legendre equation removes Y''):
        Ia = 2pi [ v^2 B_p' B_r' B_k A1 + B_p B_r B_k A2 ]
        Ib =  pi [ v^2 B_p'' B_r'' G0 + 2 (B_p' - B_p/v)(B_r' - B_r/v) G1 + 2 B_p' B_r' G0
                   + B_p' B_r / v (G2 - G5) + B_p B_r' / v (G3 - G6) + B_p B_r / v^2 (G4 + G7) ] B_k
    A1 = <Yq Ys Yl>, A2 = <a Yq' Ys' Yl>, G0 = A1, G1 = A2, G2 = <Yq Zs Yl>,
    G3 = <Zq Ys Yl>, G4 = <Zq Zs Yl>, G5 = <Yq mu Ys' Yl>, G6 = <mu Yq' Ys Yl>,
    G7 = <mu^2 Yq' Ys' Yl>, <.> = int_{-1}^{1} dmu.

    Returns (triples, A[t, 2], G[t, 6]) where A = (A1, A2) and
    G = (G0, G1, G2 - G5, G3 - G6, G4 + G7, unused 0) for each kept triple t = (q, l, s).
    """
    if nq is None:
        nq = 3 * l_max + 8
    mu, w = np.polynomial.legendre.leggauss(nq)
    L = l_max + 1
    Y = np.zeros((L, nq))
    dY = np.zeros((L, nq))
    for l in range(L):
        c = np.zeros(l + 1)
        c[l] = 1.0
        Y[l] = np.polynomial.legendre.legval(mu, c) * sph_harm_norm(l)
        dY[l] = np.polynomial.legendre.legval(mu, np.polynomial.legendre.legder(c)) * sph_harm_norm(l)
    Z = np.array([mu * dY[l] - l * (l + 1) * Y[l] for l in range(L)])
    a = 1.0 - mu * mu
    triples, A, G = [], [], []
    for q in range(L):
        for l in range(L):
            for s in range(L):
                yl = Y[l] * w
                A1 = np.sum(Y[q] * Y[s] * yl)
                A2 = np.sum(a * dY[q] * dY[s] * yl)
                G2 = np.sum(Y[q] * Z[s] * yl)
                G3 = np.sum(Z[q] * Y[s] * yl)
                G4 = np.sum(Z[q] * Z[s] * yl)
                G5 = np.sum(Y[q] * mu * dY[s] * yl)
                G6 = np.sum(mu * dY[q] * Y[s] * yl)
                G7 = np.sum(mu * mu * dY[q] * dY[s] * yl)
                vals = np.array([A1, A2, G2 - G5, G3 - G6, G4 + G7])
                if np.max(np.abs(vals)) > 1e-13:
                    triples.append((q, l, s))
                    A.append([A1, A2])
                    G.append([A1, A2, G2 - G5, G3 - G6, G4 + G7, 0.0])
    return triples, np.array(A), np.array(G)


class Operators:
    """Everything `bte_0d3v_batched.assemble_operators` builds for one v-space grid
    (bte_0d3v_batched.py:310-479), with `vspace_ext` NONE or LINEAR and CG splines."""

    def __init__(self, processes, ev_max, Te, n_sp, l_max, sp_order=3, spline_qpts=5,
                 extend_linear=False, ee=True, dense_coulomb=True, snap=True):
        self.processes = processes
        self.sp_order = sp_order
        self.num_p = n_sp
        self.lm = [[l, 0] for l in range(l_max + 1)]
        self.num_sh = len(self.lm)
        self.n = n_sp * self.num_sh
        self.vth = float(electron_thermal_velocity(Te * TEMP_K_1EV))
        vth = self.vth
        self.mw0 = 1.0 / ((vth * np.sqrt(np.pi)) ** 3)  # utils.py:713-715 at x=0

        sig = sorted(set([g.threshold for g in processes if g.threshold is not None and g.threshold > 0]))
        self.sig_pts = np.array(sig)
        dg_nodes = np.sqrt(self.sig_pts) * C_GAMMA / vth
        k_domain = (0.0, np.sqrt(ev_max) * C_GAMMA / vth)
        dom = (k_domain[0], 1.2 * k_domain[1]) if extend_linear else k_domain
        t = uniform_knots(dom, n_sp, sp_order)
        if snap:  # the 1D3V solver's basis has no threshold knots (bte_1d3v_solver.py:356)
            t = snap_knots(t, k_domain, sp_order, dg_nodes)
        self.knots = t
        self.k_domain = k_domain
        self.basis = B = Basis(t, sp_order)
        self.num_q_radial = B.num_intervals * spline_qpts

        self._assemble_mass()
        self._assemble_collisions()
        self._assemble_qoi_ops()
        self._assemble_advection()
        n = self.n
        self.op_advection = self.Minv @ self.adv_raw * (1.0 / vth) * QE_BY_ME       # :421
        self.op_col_en = np.array([self.Minv @ F for F in self.FOp])                  # :422
        self.op_col_gT = self.Minv @ self.FOp_g                                       # :423
        u = self.op_mass * self.mw0 * vth ** 3                                         # :425-428
        self.u = u
        p_vec = u.reshape((n, 1)) / np.sqrt(np.dot(u, u))
        Qm, Rm = np.linalg.qr(np.eye(n) - np.outer(p_vec, p_vec))                      # :432-433
        drop = (self.num_p - 1) * self.num_sh + 0                                       # :439-440
        self.Qmat = np.delete(Qm, drop, axis=1)
        self.Rmat = np.delete(Rm, drop, axis=0)
        self.ee = ee
        if ee:
            self._assemble_rosenbluth()
            self._assemble_coulomb(dense=dense_coulomb)

    # -- mass (spec_spherical.py:226-277) and its Cholesky inverse (:299-336)
    def _assemble_mass(self):
        B = self.basis
        gx, gw = B.gauss_pn(2 * (self.sp_order + 2) * B.num_intervals)
        V = B.vandermonde(gx)
        mm = np.zeros((self.num_p, self.num_p))
        for p in range(self.num_p):
            msk = B.support_mask(p, gx)
            for k in range(max(0, p - (self.sp_order + 3)), min(self.num_p, p + (self.sp_order + 3))):
                mm[p, k] = np.dot(gx[msk] ** 2 * V[p, msk] * V[k, msk], gw[msk])
        self.mass_radial = mm
        self.Mmat = _place_blocks(lambda l: mm, self.lm, self.num_p)
        L = np.linalg.cholesky(self.Mmat)
        Linv = scipy.linalg.solve_triangular(L, np.identity(self.n), lower=True)
        self.Minv = Linv.T @ Linv

    # -- electron-heavy collisions (collision_operator_spherical.py:79-225) and the
    #    gas-temperature term (:443-498); summed per species (bte_0d3v_batched.py:370-386)
    def _assemble_collisions(self):
        B, vth = self.basis, self.vth
        gx, gw = B.gauss_pn(self.num_q_radial)
        species = []
        for g in self.processes:
            if g.species not in species:
                species.append(g.species)
        self.species = species
        Vx = B.vandermonde(gx)
        Dx = B.vandermonde(gx, 1)
        FOp = [np.zeros((self.n, self.n)) for _ in species]
        FOp_g = np.zeros((self.n, self.n))
        for g in self.processes:
            q0, q1 = self._collision_radial(g, gx, gw, Vx)
            FOp[species.index(g.species)] += _place_blocks(lambda l: q0 if l == 0 else q1, self.lm, self.num_p)
            if g.gtype == 0:
                sig = g.total_cross_section((gx * vth / C_GAMMA) ** 2)
                kappa = (KB * 1.0 * 2 * g.mByM * 0.5 / ME) / vth
                w = gw * (-kappa) * gx ** 3 * sig
                qT = np.zeros((self.num_p, self.num_p))
                for k in range(self.num_p):
                    msk = B.support_mask(k, gx)
                    qT[:, k] = (Dx[:, msk] * (w[msk] * Dx[k, msk])).sum(axis=1)
                FOp_g += _place_blocks(lambda l: qT if l == 0 else None, self.lm, self.num_p)
        self.FOp = FOp
        self.FOp_g = FOp_g

    def _collision_radial(self, g, gx, gw, Vx):
        B, vth = self.basis, self.vth
        if g.gtype == 0:
            sig = g.total_cross_section((gx * vth / C_GAMMA) ** 2)
            vpost = gx * np.sqrt(1.0 - 2.0 * g.mByM)
            xs, ws, Vxs, split = gx, gw, Vx, 1.0
        else:
            split = 2.0 if g.gtype == 2 else 1.0
            if g.gtype in (1, 2):
                keep = (gx * vth / C_GAMMA) ** 2 >= g.threshold
                xs, ws, Vxs = gx[keep], gw[keep], Vx[:, keep]
                vpost = C_GAMMA * np.sqrt((1.0 / split) * ((xs * vth / C_GAMMA) ** 2 - g.threshold)) / vth
            else:
                xs, ws, Vxs = gx, gw, Vx
                vpost = C_GAMMA * np.sqrt((1.0 / split) * ((xs * vth / C_GAMMA) ** 2 + g.attachment_energy)) / vth
            sig = g.total_cross_section((xs * vth / C_GAMMA) ** 2)
        Vp = B.vandermonde(vpost)
        base = vth * xs ** 3 * sig * ws
        q0 = np.zeros((self.num_p, self.num_p))
        q1 = np.zeros((self.num_p, self.num_p))
        for k in range(self.num_p):
            msk = B.support_mask(k, xs)
            wk = base[msk] * Vxs[k, msk]
            q0[:, k] = ((split * Vp[:, msk] - Vxs[:, msk]) * wk).sum(axis=1)
            q1[:, k] = (-Vxs[:, msk] * wk).sum(axis=1)
        return q0, q1

    # -- QoI functionals (utils.py:73-150, 321-395, 854-944; bte_0d3v_batched.py:390-400)
    def _radial_functional(self, deg, weight):
        B = self.basis
        gx, gw = B.gauss_pn(deg)
        V = B.vandermonde(gx)
        wv = weight(gx)
        out = np.zeros(self.num_p)
        for p in range(self.num_p):
            msk = B.support_mask(p, gx)
            out[p] = np.dot(gw[msk], wv[msk] * V[p, msk])
        return out

    def _assemble_qoi_ops(self):
        B, vth = self.basis, self.vth
        ni = B.num_intervals
        sph_fac = sph_harm_norm(0) * 4 * np.pi
        m = self._radial_functional(2 * (self.sp_order + 2) * ni, lambda x: x ** 2)
        self.op_mass = np.zeros(self.n)
        self.op_mass[0::self.num_sh] = sph_fac * m
        tt = self._radial_functional(2 * (self.sp_order + 3) * ni, lambda x: x ** 4)
        self.op_temp = np.zeros(self.n)
        self.op_temp[0::self.num_sh] = sph_fac * tt
        self.op_temp = self.op_temp * 0.5 * ME * (2 / 3 / KB) / TEMP_K_1EV
        self.op_mobility = (2 * vth ** 4 / C_GAMMA ** 4) * self._radial_functional(
            2 * (self.sp_order + 3) * ni, lambda x: x ** 3)
        gx, gw = B.gauss_pn(self.num_q_radial)
        tot = 0
        for g in self.processes:
            tot = tot + g.total_cross_section((gx * vth / C_GAMMA) ** 2)
        V = B.vandermonde(gx)
        self.op_diffusion = np.zeros(self.num_p)
        for p in range(self.num_p):
            msk = B.support_mask(p, gx)
            self.op_diffusion[p] = (2 * vth ** 4 / C_GAMMA ** 4) * np.dot(gw[msk], gx[msk] ** 3 * V[p, msk] / tot[msk])
        self.op_rate = []
        for g in self.processes:
            sg = g.total_cross_section((gx * vth / C_GAMMA) ** 2)
            r = np.zeros(self.num_p)
            for p in range(self.num_p):
                msk = B.support_mask(p, gx)
                r[p] = (2 * vth ** 4 / C_GAMMA ** 3) * np.dot(gw[msk], gx[msk] ** 3 * sg[msk] * V[p, msk])
            self.op_rate.append(r)
        self.op_rate = np.array(self.op_rate)

    # -- CG advection (spec_spherical.py:432-500)
    def _assemble_advection(self):
        B = self.basis
        gx, gw = B.gauss_pn((self.sp_order + 2) * 2 * B.num_intervals)
        V = B.vandermonde(gx)
        D = B.vandermonde(gx, 1)
        mm1 = np.zeros((self.num_p, self.num_p))
        mm2 = np.zeros((self.num_p, self.num_p))
        for p in range(self.num_p):
            msk = B.support_mask(p, gx)
            for k in range(max(0, p - (self.sp_order + 3)), min(self.num_p, p + (self.sp_order + 3))):
                mm1[p, k] = np.dot(gx[msk] ** 2 * V[p, msk] * D[k, msk], gw[msk])
                mm2[p, k] = np.dot(gx[msk] * V[p, msk] * V[k, msk], gw[msk])
        num_sh = self.num_sh
        adv = np.zeros((self.num_p, num_sh, self.num_p, num_sh))
        for qi, (q, _) in enumerate(self.lm):
            if q + 1 <= self.lm[-1][0]:
                l = q + 1
                adv[:, qi, :, l] = mm1 * AM(l) + AD(l) * mm2
            if q - 1 >= 0:
                l = q - 1
                adv[:, qi, :, l] = mm1 * BM(l) + BD(l) * mm2
        self.adv_mm1, self.adv_mm2 = mm1, mm2
        self.adv_raw = adv.reshape(self.n, self.n)

    # -- Rosenbluth potential operators (collision_operator_spherical.py:786-971)
    def _assemble_rosenbluth(self):
        B, k_vec, sp = self.basis, self.knots, self.sp_order
        gmx, gmw = B.gauss_pn(self.num_q_radial)
        num_p = self.num_p

        def integrate(m, i, xb, xe, qx_e, qw_e):
            q_int = 0.0
            for kn in range(i + 1, i + sp + 2):
                a = max(xb, k_vec[kn - 1])
                b = min(xe, k_vec[kn])
                if b > a:
                    qx = 0.5 * ((b - a) * qx_e + (b + a))
                    qw = 0.5 * (b - a) * qw_e
                    q_int += np.dot(qw, (qx ** m) * B.eval(i, qx))
            return q_int

        def Pm(m):
            qo = (((sp + abs(m) + 1) // 2) + 1) * 4
            qx, qw = np.polynomial.legendre.leggauss(qo)
            pm = np.zeros((num_p, len(gmx)))
            for i in range(num_p):
                idx = np.where((k_vec[i] <= gmx) & (gmx <= k_vec[i + sp + 1]))[0]
                for j in idx:
                    pm[i, j] = integrate(m, i, k_vec[i], gmx[j], qx, qw)
                after = np.where(k_vec[i + sp + 1] < gmx)[0]
                pm[i, after] = integrate(m, i, k_vec[i], k_vec[i + sp + 1], qx, qw)
            return pm

        def Qm(m):
            qo = (((sp + abs(m) + 1) // 2) + 1) * 32
            qx, qw = np.polynomial.legendre.leggauss(qo)
            qm = np.zeros((num_p, len(gmx)))
            for i in range(num_p):
                idx = np.where((k_vec[i] <= gmx) & (gmx <= k_vec[i + sp + 1]))[0]
                for j in idx:
                    qm[i, j] = integrate(-m, i, gmx[j], k_vec[i + sp + 1], qx, qw)
                before = np.where(gmx < k_vec[i])[0]
                qm[i, before] = integrate(-m, i, k_vec[i], k_vec[i + sp + 1], qx, qw)
            return qm

        cacheP, cacheQ = {}, {}

        def P(m):
            if m not in cacheP:
                cacheP[m] = Pm(m)
            return cacheP[m]

        def Qf(m):
            if m not in cacheQ:
                cacheQ[m] = Qm(m)
            return cacheQ[m]

        m_ab = 1.0
        Vq = B.vandermonde(gmx)
        W = gmx ** 2 * gmw
        hl_op = np.zeros((self.n, self.n))
        gl_op = np.zeros((self.n, self.n))
        self.ros_m1, self.ros_m2 = [], []
        for li, (ll, _) in enumerate(self.lm):
            f1 = (ll - 0.5) / (ll + 1.5)
            m1 = (2 / (2 * ll + 1)) * (1 + m_ab) * (P(ll + 2) / (gmx ** (ll + 1)) + Qf(ll - 1) * gmx ** ll)
            m2 = -(2 / (4 * ll ** 2 - 1)) * ((P(ll + 2) / gmx ** (ll - 1) - f1 * P(ll + 4) / gmx ** (ll + 1))
                                            + (Qf(ll - 3) * gmx ** ll - f1 * Qf(ll - 1) * gmx ** (ll + 2)))
            self.ros_m1.append(m1)
            self.ros_m2.append(m2)
            hl_op[li::self.num_sh, li::self.num_sh] = (Vq * W) @ m1.T
            gl_op[li::self.num_sh, li::self.num_sh] = (Vq * W) @ m2.T
        self.hl_raw, self.gl_raw = hl_op, gl_op
        self.hl_op = self.Minv @ hl_op
        self.gl_op = self.Minv @ gl_op

    # -- Coulomb trilinear forms (collision_operator_spherical.py:973-1120) and their
    #    contraction with the potentials (bte_0d3v_batched.py:444-476)
    def _assemble_coulomb(self, dense=True):
        B, sp, num_p, num_sh = self.basis, self.sp_order, self.num_p, self.num_sh
        l_max = self.lm[-1][0]
        gmx, gmw = B.gauss_pn(self.num_q_radial)
        V = [B.vandermonde(gmx, d) for d in range(3)]
        triples, A, G = coulomb_angular_tables(l_max)
        self.cc_triples, self.cc_A, self.cc_G = triples, A, G
        band = sp  # nonzero only where all three supports overlap: |p-k|, |p-r|, |k-r| <= sp
        nb = 2 * band + 1
        Ra = np.zeros((num_p, nb, nb, 2))
        Rb = np.zeros((num_p, nb, nb, 6))
        inv_v = 1.0 / gmx
        for p in range(num_p):
            for dk in range(-band, band + 1):
                k = p + dk
                if k < 0 or k >= num_p:
                    continue
                for dr in range(-band, band + 1):
                    r = p + dr
                    if r < 0 or r >= num_p or abs(k - r) > band:
                        continue
                    kmin = min(self.knots[p], self.knots[k], self.knots[r])
                    kmax = max(self.knots[p + sp + 1], self.knots[k + sp + 1], self.knots[r + sp + 1])
                    msk = (gmx >= kmin) & (gmx <= kmax)
                    w, x, iv = gmw[msk], gmx[msk], inv_v[msk]
                    Bp, Dp, DDp = V[0][p, msk], V[1][p, msk], V[2][p, msk]
                    Bk = V[0][k, msk]
                    Br, Dr, DDr = V[0][r, msk], V[1][r, msk], V[2][r, msk]
                    wk = w * Bk
                    Ra[p, dk + band, dr + band, 0] = np.dot(wk, x * x * Dp * Dr)
                    Ra[p, dk + band, dr + band, 1] = np.dot(wk, Bp * Br)
                    Rb[p, dk + band, dr + band, 0] = np.dot(wk, x * x * DDp * DDr)
                    Rb[p, dk + band, dr + band, 1] = np.dot(wk, (Dp - Bp * iv) * (Dr - Br * iv))
                    Rb[p, dk + band, dr + band, 2] = np.dot(wk, Dp * Dr)
                    Rb[p, dk + band, dr + band, 3] = np.dot(wk, Dp * Br * iv)
                    Rb[p, dk + band, dr + band, 4] = np.dot(wk, Bp * Dr * iv)
                    Rb[p, dk + band, dr + band, 5] = np.dot(wk, Bp * Br * iv * iv)
        self.cc_Ra, self.cc_Rb = Ra, Rb
        if dense:
            n = self.n
            cca = np.zeros((n, n, n))
            ccb = np.zeros((n, n, n))
            for p in range(num_p):
                for dk in range(-band, band + 1):
                    k = p + dk
                    if k < 0 or k >= num_p:
                        continue
                    for dr in range(-band, band + 1):
                        r = p + dr
                        if r < 0 or r >= num_p or abs(k - r) > band:
                            continue
                        ra = Ra[p, dk + band, dr + band]
                        rb = Rb[p, dk + band, dr + band]
                        for ti, (q, l, s) in enumerate(triples):
                            a = 2 * np.pi * (ra[0] * A[ti, 0] + ra[1] * A[ti, 1])
                            g = G[ti]
                            b = np.pi * (rb[0] * g[0] + 2 * rb[1] * g[1] + 2 * rb[2] * g[0]
                                         + rb[3] * g[2] + rb[4] * g[3] + rb[5] * g[4])
                            cca[p * num_sh + q, k * num_sh + l, r * num_sh + s] = a
                            ccb[p * num_sh + q, k * num_sh + l, r * num_sh + s] = b
            self.cc_a, self.cc_b = cca, ccb
            cc = np.dot(cca, self.hl_op) + np.dot(ccb, self.gl_op)
            cc = np.dot(self.Minv, cc.reshape((n, -1))).reshape((n, n, n))
            self.cc_op = cc


# ----------------------------------------------------------------------------------
# Steady-state solve (bte_0d3v_batched.py:602-979, 1163-1217)
# ----------------------------------------------------------------------------------
class Params:
    def __init__(self, n0, ne, Tg, E, ns_by_n0):
        self.n0 = np.asarray(n0, dtype=np.float64)
        self.ne = np.asarray(ne, dtype=np.float64)
        self.Tg = np.asarray(Tg, dtype=np.float64)
        self.E = np.asarray(E, dtype=np.float64)
        self.ns_by_n0 = np.asarray(ns_by_n0, dtype=np.float64)


def rhs_and_jacobian(ops: Operators, prm: Params, ee: bool):
    """get_rhs_and_jacobian, bte_0d3v_batched.py:602-821 (dg off, qA = I)."""
    vth, mw0 = ops.vth, ops.mw0
    Mop = ops.op_mass.reshape((1, -1))
    Top = ops.op_temp.reshape((1, -1)) * TEMP_K_1EV
    Q, QT = ops.Qmat, ops.Qmat.T
    c_en, c_gT, adv = ops.op_col_en, ops.op_col_gT, ops.op_advection
    u = ops.u
    Wmat = np.einsum("v,svu->su", u, c_en)
    QT_Cen = np.einsum("mu,suv->smv", QT, c_en)
    QT_Cgt = QT @ c_gT
    QT_A = QT @ adv
    QT_Cen_Q = np.einsum("av,svu->sau", QT, np.dot(c_en, Q))
    QT_Cgt_Q = QT @ (c_gT @ Q)
    QT_A_Q = QT @ (adv @ Q)
    Imat = np.eye(QT.shape[0])
    n0, ne, Tg, E, ns_by_n0 = prm.n0, prm.ne, prm.Tg, prm.E, prm.ns_by_n0

    def gamma_a(fb):
        m0 = mw0 * np.dot(Mop, fb) * vth ** 3
        kT = mw0 * (np.dot(Top, fb) / m0) * vth ** 5 * KB
        kT = np.abs(kT).reshape((-1,))
        c_lambda = ((12 * np.pi * (EPS0 * kT) ** 1.5) / (QE ** 3 * np.sqrt(ne)))
        return (np.log(c_lambda) * QE ** 4) / (4 * np.pi * (EPS0 * ME) ** 2) / vth ** 3

    def res(x):
        y = (n0 * (np.einsum("sx,svx->vx", ns_by_n0, np.dot(QT_Cen, x)) + Tg * np.dot(QT_Cgt, x))
             + E * np.dot(QT_A, x)
             - n0 * np.einsum("sx,sx->x", ns_by_n0, np.dot(Wmat, x)) * np.dot(QT, x))
        if ee:
            c_ee_x = np.dot(ops.cc_op, x)
            c_ee_xx = np.einsum("abc,bc->ac", c_ee_x, x)
            y = y + ne * gamma_a(x) * np.dot(QT, c_ee_xx)
        return y

    def jac(x):
        ns = n0 * ns_by_n0
        L = np.einsum("sx,svu->xvu", ns, QT_Cen_Q) + np.einsum("a,bc->abc", n0 * Tg, QT_Cgt_Q)
        mu = np.einsum("sx,sx->x", ns, np.dot(Wmat, x))
        L = L + np.einsum("a,bc->abc", E, QT_A_Q) - np.einsum("a,bc->abc", mu, Imat)
        if ee:
            cc = np.dot(ops.cc_op, x) + np.dot(np.swapaxes(ops.cc_op, 1, 2), x)
            cc = np.swapaxes(np.swapaxes(cc, 0, 2), 1, 2)
            ccQ = np.einsum("abc,cd->abd", cc, Q)
            QTccQ = np.einsum("be,aec->abc", QT, ccQ)
            L = L + np.einsum("a,abc->abc", ne * gamma_a(x), QTccQ)
        return L

    return res, jac, gamma_a


def normalized_distribution(ops: Operators, ff):
    """bte_0d3v_batched.py:1204-1217."""
    mm_fac = sph_harm_norm(0) * 4 * np.pi
    scale = np.dot(ops.op_mass / mm_fac, ff) * (2 * (ops.vth / C_GAMMA) ** 3)
    return ff / scale


def compute_qois(ops: Operators, prm: Params, ff, effective_mobility=True):
    """bte_0d3v_batched.py:1163-1202."""
    vth, mw0, nsh = ops.vth, ops.mw0, ops.num_sh
    mm = np.dot(ops.op_mass, ff) * mw0 * vth ** 3
    mu = 1.5 * np.dot(ops.op_temp, ff) * mw0 * vth ** 5 / mm
    if effective_mobility:
        M = np.dot(ops.op_mobility, np.sqrt(3) * ff[1::nsh, :]) * (-(C_GAMMA / (3 * (prm.E / prm.n0))))
    else:
        M = np.dot(ops.op_mobility, np.sqrt(3) * ff[1::nsh, :]) * (-(C_GAMMA / (3 * (1 / prm.n0))))
    D = np.dot(ops.op_diffusion, ff[0::nsh, :]) * (C_GAMMA / 3.0)
    rr = np.array([np.dot(r, ff[0::nsh, :]) for r in ops.op_rate])
    return {"energy": mu, "mobility": M, "diffusion": D, "rates": rr}


def maxwellian_initial(ops: Operators, n_pts):
    """initialize(..., "maxwellian"), bte_0d3v_batched.py:481-520, through
    utils.function_to_basis (utils.py:475-532) with 2 theta and 2 phi points."""
    B = ops.basis
    gmx, gmw = B.gauss_pn(ops.num_q_radial)
    glx, glw = np.polynomial.legendre.leggauss(2)
    vt = np.arccos(glx)
    wvp = (2 * np.pi / 2) * np.ones(2)
    hq = (1 / np.sqrt(np.pi) ** 3) * np.exp(-gmx ** 2) * gmx ** 2
    V = B.vandermonde(gmx)
    radial = V @ (hq * gmw)  # (num_p,)
    h = np.zeros(ops.n)
    for li, (l, _) in enumerate(ops.lm):
        c = np.zeros(l + 1)
        c[l] = 1
        Yl = sph_harm_norm(l) * np.polynomial.legendre.legval(np.cos(vt), c)
        ang = np.sum(Yl * glw) * np.sum(wvp)
        h[li::ops.num_sh] = radial * ang
    h = ops.Minv @ h
    return np.repeat(h[:, None], n_pts, axis=1)


def steady_state_solve(ops: Operators, prm: Params, f0, atol, rtol, max_iter, ee,
                       alpha_min=1e-16, alpha_rho=0.01, line_search_c=1e-3, log=None):
    """steady_state_solve, bte_0d3v_batched.py:882-979 (the batch-global loop, per-point
    Armijo backtracking and final normalisation). Returns (ff, qoi, info)."""
    gen = steady_state_iterations(ops, prm, f0, atol, rtol, max_iter, ee, alpha_min, alpha_rho, line_search_c, log)
    while True:
        try:
            next(gen)
        except StopIteration as stop:
            return stop.value


def steady_state_iterations(ops: Operators, prm: Params, f0, atol, rtol, max_iter, ee,
                            alpha_min=1e-16, alpha_rho=0.01, line_search_c=1e-3, log=None):
    """steady_state_solve as a generator that yields after every Newton iteration of the
    batch-global loop (so a caller can time bounded slices of one solve) and returns
    (ff, qoi, info) when the reference's loop would end."""
    n_pts = f0.shape[1]
    u = ops.u
    Q, R = ops.Qmat, ops.Rmat
    res, jac, _ = rhs_and_jacobian(ops, prm, ee)
    f0 = f0 / np.dot(u, f0)
    fb_prev = np.dot(R, f0)
    f1 = u / np.dot(u, u)
    h_prev = f1[:, None] + np.dot(Q, fb_prev)
    r0 = np.linalg.norm(res(h_prev), axis=0, ord=2)
    abs_error = r0.copy()
    it = 0
    n_res = 1  # residual evaluations (the line search's trial steps dominate late iterations)
    h_curr = h_prev
    status = "max_iter"
    while (abs_error > atol + rtol * r0).any() and it < max_iter:
        L = jac(h_prev)
        rhs_vec = res(h_prev)
        abs_error = np.linalg.norm(rhs_vec, axis=0, ord=2)
        Linv = np.linalg.inv(L)
        pp = np.einsum("abc,ca->ba", Linv, -rhs_vec)
        p = np.dot(Q, pp)
        alpha = np.ones(n_pts)
        diverged = False
        rf_new = 0.5 * np.linalg.norm(res(h_prev + alpha * p), axis=0, ord=2) ** 2
        n_res += 2
        while (rf_new > 0.5 * abs_error ** 2 - line_search_c * alpha * abs_error ** 2).any():
            rc = rf_new > 0.5 * abs_error ** 2 - line_search_c * alpha * abs_error ** 2
            alpha[rc] *= alpha_rho
            if (alpha < alpha_min).all():
                diverged = True
                break
            rf_new = 0.5 * np.linalg.norm(res(h_prev + alpha * p), axis=0, ord=2) ** 2
            n_res += 1
        if diverged:
            status = "line_search"
            break
        h_curr = h_prev + alpha * p
        if it % 10 == 0:
            abs_error = np.linalg.norm(res(h_curr), axis=0)
            n_res += 1
            if log:
                log(it, abs_error, abs_error / r0)
        h_prev = h_curr
        it += 1
        yield it
    else:
        status = "converged" if not (abs_error > atol + rtol * r0).any() else "max_iter"
    abs_error = np.linalg.norm(res(h_curr), axis=0)
    ff = normalized_distribution(ops, h_curr)
    qoi = compute_qois(ops, prm, ff, effective_mobility=True)
    return ff, qoi, dict(iters=it, abs_error=abs_error, rel_error=abs_error / r0, status=status, res_evals=n_res)


def processes_from_lxcat(path):
    """bte_0d3v_batched.py:197-221: one Process per block, m/M from the elastic argon key."""
    import os
    import sys
    sys.path.insert(0, os.path.abspath(os.path.join(os.path.dirname(__file__), "..")))
    from boltzmann_gb300.lxcat import read_cross_section_data
    data = read_cross_section_data(path)
    mByM = data["E + Ar -> E + Ar"]["mass_ratio"]
    return [Process(k, v, mByM) for k, v in data.items()]


def transient_solve(ops: Operators, prm: Params, f0, dt, cycles, efreq, eRe, eIm, atol, rtol, max_iter, ee):
    """solve(..., "transient"), bte_0d3v_batched.py:1063-1155, with newton_solver_batched
    (:59-126): backward Euler in the mass-conserving coordinates du (u + Q du), the Jacobian
    frozen at the step's start and inverted once (a chord iteration, no line search), the
    batch stopping when all points meet rtol or all meet atol; t is in RF periods and
    tau = 1 / efreq (1e-7 without a field frequency); E(t) = eRe cos 2 pi t + eIm sin 2 pi t
    when efreq > 0. Returns (u, qoi of the last completed cycle average, info)."""
    vth = ops.vth
    tau = 1e-7 if efreq == 0 else 1.0 / efreq
    io_freq = int(1.0 / dt)
    steps_total = int(cycles / dt)
    Q = ops.Qmat
    u = f0 / np.dot(ops.u, f0)
    P = f0.shape[1]
    m = Q.shape[1]
    du = np.zeros((m, P))
    cyc = np.zeros_like(u)
    cyc_v = np.zeros_like(u)
    I = np.eye(m)
    tt = 0.0
    iters = []
    for ts in range(steps_total + 1):
        E = (eRe * np.cos(2 * np.pi * (tt + dt)) + eIm * np.sin(2 * np.pi * (tt + dt))) if efreq > 0 else prm.E
        pt = Params(prm.n0, prm.ne, prm.Tg, E, prm.ns_by_n0)
        res, jac, _ = rhs_and_jacobian(ops, pt, ee)
        J = np.einsum("i,jk->ijk", np.ones(P), I) - dt * tau * jac(u)
        Jinv = np.linalg.inv(J)
        x = du
        r0n = np.linalg.norm(x - dt * tau * res(u + Q @ x), axis=0)
        count = 0
        converged = False
        while True:
            rr = x - dt * tau * res(u + Q @ x)
            rn = np.linalg.norm(rr, axis=0)
            converged = bool(np.all(rn / r0n < rtol) or np.all(rn < atol))
            if converged or count >= max_iter:
                break
            x = x + np.einsum("ijk,ki->ji", Jinv, -rr)
            count += 1
        iters.append(count)
        if not converged:
            raise RuntimeError("transient Newton step did not converge at t = %.3e" % tt)
        if ts > 0 and ts % io_freq == 0:
            cyc *= 0.5 * dt
            cyc_v = cyc.copy()
            cyc[:] = 0
            if ts == steps_total:
                break
        cyc += u
        du = x
        u = u + Q @ du
        cyc += u
        tt += dt
    h = normalized_distribution(ops, cyc_v)
    E_last = prm.E
    qoi = compute_qois(ops, Params(prm.n0, prm.ne, prm.Tg, E_last, prm.ns_by_n0), h, effective_mobility=False)
    return u, qoi, dict(iters=np.array(iters), cycle_avg=h)
