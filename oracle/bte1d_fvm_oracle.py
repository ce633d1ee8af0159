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

import math

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


# ----------------------------------------------------------------------------------
# Set-up: the FVM v-grid and the electron-heavy collision operator on it
# ----------------------------------------------------------------------------------
def fvm_vr_grid(basis, spline_qpts):
    """Radial FVM cells: the B-spline basis's per-interval Gauss-Legendre points and weights
    (spec_spherical.gl_vr with use_bspline_qgrid, spec_spherical.py:1010-1012)."""
    return basis.gauss_pn(spline_qpts * basis.num_intervals)


def _linear_weights(xs, grid):
    """Rows: the linear-interpolation weights of the grid values at xs, zero outside
    [grid[0], grid[-1]] (scipy interp1d, kind linear, fill 0)."""
    W = np.zeros((len(xs), len(grid)))
    for k in range(len(grid)):
        e = np.zeros(len(grid))
        e[k] = 1.0
        W[:, k] = np.interp(xs, grid, e, left=0.0, right=0.0)
    return W


def collision_op_fvm(processes, vr, vr_qw, vt, vt_qw, vth, rmax, c_gamma):
    """Sum over processes of the strong-form binary collision operator on the (v_r, theta) FVM
    grid, index r * Nvt + j (collision_operator_spherical.py:1334-1437):
      C f = (gain) - (loss),  loss_r = 4 pi s(v_r), s(v) = v vth sigma(eps(v)) / (4 pi),
      gain_r = s(v_pre) J(v_r) * [f interpolated at v_pre(v_r)] averaged over theta,
    with v_pre and J per process: elastic v / sqrt(1 - 2 m/M), J = (1 - 2 m/M)^(-3/2);
    excitation sqrt(v^2 + (c_gamma/vth)^2 eps_th), J = v_pre / v; ionization
    sqrt(2 v^2 + (c_gamma/vth)^2 eps_th), J = 4 v_pre / v. Interpolation is linear on the
    v_r cells, zero below the first cell, and falls linearly from the last cell to 0 at
    rmax."""
    nr, nt = len(vr), len(vt)
    eps = lambda v: (v * vth / c_gamma) ** 2
    avg = np.tile(2.0 * np.pi * np.asarray(vt_qw), (nt, 1))   # each row: the theta average
    F = np.zeros((nr * nt, nr * nt))
    for g in processes:
        if g.gtype == 0:
            scale = math.sqrt(1.0 - 2.0 * g.mByM)
            vpre = vr / scale
            J = np.full(nr, scale ** -3)
        elif g.gtype == 1:
            vpre = np.sqrt(vr ** 2 + (c_gamma / vth) ** 2 * g.threshold)
            J = vpre / vr
        elif g.gtype == 2:
            vpre = np.sqrt(2.0 * vr ** 2 + (c_gamma / vth) ** 2 * g.threshold)
            J = 4.0 * vpre / vr
        else:
            raise NotImplementedError("attachment has no strong-form FVM operator in the reference")
        s = vr * vth * g.total_cross_section(eps(vr)) / (4.0 * np.pi)
        s_pre = vpre * vth * g.total_cross_section(eps(vpre)) / (4.0 * np.pi)
        Lw = _linear_weights(vpre, vr)
        tail = (vpre > vr[-1]) & (vpre <= rmax)
        Lw[tail, -1] = (rmax - vpre[tail]) / (rmax - vr[-1])
        F += np.kron(np.diag(s_pre * J) @ Lw, avg) - 4.0 * np.pi * np.kron(np.diag(s), np.eye(nt))
    return F


def collision_inverse(F, dt, tau, n0, np0):
    """PmatC = (I - dt tau n0 np0 F)^-1, the op-split step's collision solve
    (bte_1d3v_solver.py:1346-1375; no gas-temperature term on the FVM grid)."""
    return np.linalg.inv(np.eye(F.shape[0]) - dt * tau * n0 * np0 * F)


# ----------------------------------------------------------------------------------
# Set-up: upwind first-derivative operators and their band arrays
# ----------------------------------------------------------------------------------
def _lagrange_d1(xs, t):
    """Weights w_k with sum_k w_k f(xs_k) = p'(t), p the interpolating polynomial of f on the
    stencil xs: w_k = l_k'(t) = sum_{m != k} 1/(x_k - x_m) prod_{j != k, m} (t - x_j)/(x_k - x_j)."""
    n = len(xs)
    w = np.zeros(n)
    for k in range(n):
        acc = 0.0
        for m in range(n):
            if m == k:
                continue
            term = 1.0 / (xs[k] - xs[m])
            for j in range(n):
                if j != k and j != m:
                    term *= (t - xs[j]) / (xs[k] - xs[j])
            acc += term
        w[k] = acc
    return w


def upwind_d1(x, sw, direction):
    """One-sided first derivative on the points x with stencils of sw points (mesh.py:20-55):
    "L" uses x[i-sw+1 .. i] (shorter near the start, row 0 empty), "R" uses x[i .. i+sw-1]
    (shorter near the end, row N-1 from the single last point: empty)."""
    N = len(x)
    D = np.zeros((N, N))
    for i in range(N):
        if direction == "L":
            lo = max(0, i - (sw - 1))
            if i > lo:
                D[i, lo:i + 1] = _lagrange_d1(x[lo:i + 1], x[i])
        else:
            hi = min(N, i + sw)
            if hi - 1 > i:
                D[i, i:hi] = _lagrange_d1(x[i:hi], x[i])
    return D


def upwind_d1_theta(x, sw, direction):
    """mesh.py:80-112 without central differences: upwind_d1 within each hemisphere of the
    ordinates, bridged by a two-point stencil across the equator (row mp for "L", row mp-1
    for "R", mp = N/2)."""
    N = len(x)
    mp = N // 2
    D = np.zeros((N, N))
    D[:mp, :mp] = upwind_d1(x[:mp], sw, direction)
    D[mp:, mp:] = upwind_d1(x[mp:], sw, direction)
    if direction == "L":
        D[mp] = 0.0
        D[mp, mp - 1:mp + 1] = _lagrange_d1(x[mp - 1:mp + 1], x[mp])
    else:
        D[mp - 1] = 0.0
        D[mp - 1, mp - 1:mp + 1] = _lagrange_d1(x[mp - 1:mp + 1], x[mp - 1])
    return D


def bands_by_column(D, nd, lower):
    """The first nd diagonals of D stored by column, as the sweeps read them: lower
    band[k][i-k] = D[i][i-k], upper band[k][i+k] = D[i][i+k] (bte_1d3v_solver.py:1452-1462)."""
    N = D.shape[0]
    B = np.zeros((nd, N))
    for k in range(nd):
        if lower:
            B[k, :N - k] = np.diagonal(D, offset=-k)
        else:
            B[k, k:] = np.diagonal(D, offset=k)
    return B


def fvm_upwind_bands(vr, vt, x, pvr, pvt, px, rmax):
    """The six band arrays of the op-split sweeps (bte_1d3v_solver.py:1406-1470): upwind
    operators of stencil width p+1; inflow rows zeroed (first row of "L", last of "R"); the
    v_r outflow row set to -1 / (rmax - v_r[-1]); theta operators scaled by sin(theta)."""
    Dvr_L, Dvr_R = upwind_d1(vr, pvr + 1, "L"), upwind_d1(vr, pvr + 1, "R")
    Dvt_L, Dvt_R = upwind_d1_theta(vt, pvt + 1, "L"), upwind_d1_theta(vt, pvt + 1, "R")
    Dx_L, Dx_R = upwind_d1(x, px + 1, "L"), upwind_d1(x, px + 1, "R")
    Dvr_L[0, :] = 0.0
    Dvr_R[-1, :] = 0.0
    Dvr_R[-1, -1] = -1.0 / (rmax - vr[-1])
    Dvt_L[0, :] = 0.0
    Dvt_R[-1, :] = 0.0
    Dx_L[0, :] = 0.0
    Dx_R[-1, :] = 0.0
    s = np.diag(np.sin(vt))
    Dvt_L, Dvt_R = s @ Dvt_L, s @ Dvt_R
    return dict(vr_diag_l2r=bands_by_column(Dvr_L, pvr + 1, True), vr_diag_r2l=bands_by_column(Dvr_R, pvr + 1, False),
                vt_diag_l2r=bands_by_column(Dvt_L, pvt + 1, True), vt_diag_r2l=bands_by_column(Dvt_R, pvt + 1, False),
                x_diag_l2r=bands_by_column(Dx_L, px + 1, True), x_diag_r2l=bands_by_column(Dx_R, px + 1, False))


# ----------------------------------------------------------------------------------
# The fully implicit step (bte_1d3v_solver.py:1890-2009)
# ----------------------------------------------------------------------------------
def adv_v_fvm(vr, vt, pvr, pvt, rmax):
    """Dense upwind v-space advection operators for E >= 0 and E < 0 (unscaled; the solver
    multiplies by qe / (me vth)), spec_spherical.py:876-951:
      A_Ep = [Dvr_RtoL on cos > 0 ordinates, Dvr_LtoR on cos < 0] (x) diag(cos) - diag(1/vr) (x) sin Dvt_RtoL,
      A_En = [Dvr_LtoR on cos > 0, Dvr_RtoL on cos < 0] (x) diag(cos)          - diag(1/vr) (x) sin Dvt_LtoR."""
    nr, nt = len(vr), len(vt)
    DL, DR = upwind_d1(vr, pvr + 1, "L"), upwind_d1(vr, pvr + 1, "R")
    TL, TR = upwind_d1_theta(vt, pvt + 1, "L"), upwind_d1_theta(vt, pvt + 1, "R")
    DL[0, :] = 0.0
    DR[-1, :] = 0.0
    DR[-1, -1] = -1.0 / (rmax - vr[-1])
    TL[0, :] = 0.0
    TR[-1, :] = 0.0
    c, s = np.cos(vt), np.sin(vt)
    pos = c > 0
    out = []
    for Dpos, Dneg, T in ((DR, DL, TR), (DL, DR, TL)):
        A = np.zeros((nr * nt, nr * nt))
        for j in range(nt):
            D = Dpos if pos[j] else Dneg
            A[j::nt, j::nt] += c[j] * D
        A -= np.kron(np.diag(1.0 / vr), np.diag(s) @ T)
        out.append(A)
    return out[0], out[1]


def x_shift_bands(vr, vt, x, px, ax, dt):
    """bte_x_shift_diag (:780-860, upwind x-space): per (r, j) the row-stored bands of
    I + dt ax v_r cos(theta_j) D, D the upwind x operator with its inflow row zeroed ("L" for
    theta <= pi/2, "R" otherwise); (Nr, Nvt, px + 1, Nx), band[k][i] = M[i][i -/+ k]."""
    Nx = len(x)
    DL, DR = upwind_d1(x, px + 1, "L"), upwind_d1(x, px + 1, "R")
    DL[0, :] = 0.0
    DR[-1, :] = 0.0
    out = np.zeros((len(vr), len(vt), px + 1, Nx))
    for j, th in enumerate(vt):
        lower = th <= 0.5 * np.pi
        D = DL if lower else DR
        for i, v in enumerate(vr):
            M = np.eye(Nx) + dt * ax * v * np.cos(th) * D
            for k in range(px + 1):
                if lower:
                    out[i, j, k, k:] = np.diagonal(M, offset=-k)
                else:
                    out[i, j, k, :Nx - k] = np.diagonal(M, offset=k)
    return out


def implicit_matvec(g, A_Ep, A_En, xshift, E, x, dt):
    """rhs_mvec (:1915-1955): y = X x - dt tau (n0 np0 C x + E (x) A_sign(E) x), the v-space part's
    inflow rows (theta <= pi/2 at the first x point, > pi/2 at the last) zeroed, X the x-shift
    bands of `x_shift_bands`. C is g["op_col_en"] (no gas-temperature term on the FVM grid);
    A_Ep, A_En already scaled by qe / (me vth)."""
    Nr, Nvt, Nx = int(g["Nr"]), int(g["Nvt"]), int(g["Nx"])
    vt = np.asarray(g["vt"])
    X = x.reshape(Nr * Nvt, Nx)
    E = np.asarray(E)
    yE = np.where(E[None, :] >= 0, A_Ep @ X, A_En @ X)
    yv = dt * float(g["tau"]) * (float(g["n0"]) * float(g["np0"]) * (np.asarray(g["op_col_en"]) @ X) + E[None, :] * yE)
    yv = yv.reshape(Nr, Nvt, Nx)
    yv[:, vt <= 0.5 * np.pi, 0] = 0.0
    yv[:, vt > 0.5 * np.pi, -1] = 0.0
    Z = X.reshape(Nr, Nvt, Nx)
    yx = np.zeros_like(Z)
    for j, th in enumerate(vt):
        yx[:, j] = SO.banded_tri_mv(xshift[:, j], Z[:, j], lower=bool(th <= 0.5 * np.pi))
    return (yx - yv).reshape(Nr * Nvt, Nx)


def implicit_rhs(g, v):
    """brhs (:1907-1911): v with the inflow values zeroed."""
    Nr, Nvt, Nx = int(g["Nr"]), int(g["Nvt"]), int(g["Nx"])
    vt = np.asarray(g["vt"])
    b = np.array(v, dtype=np.float64).reshape(Nr, Nvt, Nx)
    b[:, vt <= 0.5 * np.pi, 0] = 0.0
    b[:, vt > 0.5 * np.pi, -1] = 0.0
    return b.reshape(Nr * Nvt, Nx)


def implicit_step(g, A_Ep, A_En, xshift, E, v, dt):
    """The fully implicit step's solution, by a dense solve of rhs_mvec y = brhs (the reference
    reaches it by preconditioned GMRES to rtol): small cases only."""
    n = int(g["Nr"]) * int(g["Nvt"]) * int(g["Nx"])
    M = np.zeros((n, n))
    I = np.eye(n)
    for k in range(n):
        M[:, k] = implicit_matvec(g, A_Ep, A_En, xshift, E, I[:, k], dt).reshape(-1)
    return np.linalg.solve(M, implicit_rhs(g, v).reshape(-1)).reshape(-1, int(g["Nx"]))


# ----------------------------------------------------------------------------------
# The semi-Lagrangian step (bte_1d3v_solver.py:2024-2027, 2244-2314)
# ----------------------------------------------------------------------------------
def sl_padded(v, vr, vt, vmin):
    """The grid values padded by one layer in v_r and theta (:2282-2306): the v_r = vmin layer by
    linear extrapolation from the first two cells, the theta = pi and theta = 0 layers by linear
    extrapolation along theta (corners of the vmin layer add both terms), the v_r = vmax layer zero.
    v: (Nr, Nvt, Nx) -> (Nr + 2, Nvt + 2, Nx) with grids vrp (ascending) and vtp (pi ... 0)."""
    Nr, Nvt, Nx = v.shape
    y = np.zeros((Nr + 2, Nvt + 2, Nx))
    y[1:-1, 1:-1] = v
    dr = (vr[0] - vmin) * (v[1] - v[0]) / (vr[1] - vr[0])          # (Nvt, Nx)
    y[0, 1:-1] = v[0] - dr
    y[0, 0] = v[0, 0] - dr[0] + (np.pi - vt[0]) * (v[0, 1] - v[0, 0]) / (vt[1] - vt[0])
    y[0, -1] = v[0, -1] - dr[-1] - vt[-1] * (v[0, -1] - v[0, -2]) / (vt[-1] - vt[-2])
    y[1:-1, 0] = v[:, 0] + (np.pi - vt[0]) * (v[:, 1] - v[:, 0]) / (vt[1] - vt[0])
    y[1:-1, -1] = v[:, -1] - vt[-1] * (v[:, -1] - v[:, -2]) / (vt[-1] - vt[-2])
    return y


def sl_departure(vr, vt, x, E, dt, tau, vth, L, qe, me):
    """Departure points of each (r, j, x) value over one step (:2267-2278): x - dt tau vth / L
    v_r cos(theta), and the velocity (v_r, theta) shifted by dtE = dt tau qe / (me vth) E along
    the field axis. Returns (vr_ap, vt_ap, x_ap), each (Nr, Nvt, Nx)."""
    vrc = vr[:, None, None] * np.cos(vt)[None, :, None] * np.ones(len(x))[None, None, :]
    dtE = (dt * tau * qe / me / vth) * np.ones((len(vr), len(vt)))[:, :, None] * np.asarray(E)[None, None, :]
    x_ap = x[None, None, :] - (dt * tau * vth / L) * vrc
    vr_ap = np.sqrt((vr ** 2)[:, None, None] * np.ones((1, len(vt), len(x))) + 2 * vrc * dtE + dtE ** 2)
    vt_ap = np.arccos((vrc + dtE) / vr_ap)
    return vr_ap, vt_ap, x_ap


def _cell(grid, q):
    """Index i and fraction t with q = grid[i] + t (grid[i+1] - grid[i]), for an ascending grid;
    inside is False outside [grid[0], grid[-1]]."""
    i = np.clip(np.searchsorted(grid, q, side="left") - 1, 0, len(grid) - 2)
    t = (q - grid[i]) / (grid[i + 1] - grid[i])
    inside = (q >= grid[0]) & (q <= grid[-1])
    return i, t, inside


def sl_advect(v, vr, vt, x, E, dt, tau, vth, L, qe, me, vmin, vmax):
    """step_adv_vx_sl (:2244-2314): v (Nr * Nvt, Nx) interpolated trilinearly at the departure
    points on the padded grid, zero where a departure point leaves it."""
    Nr, Nvt, Nx = len(vr), len(vt), len(x)
    Y = sl_padded(np.asarray(v).reshape(Nr, Nvt, Nx), vr, vt, vmin)
    vrp = np.concatenate([[vmin], vr, [vmax]])
    vta = np.concatenate([[0.0], vt[::-1], [np.pi]])    # ascending theta; Y's theta axis reversed
    Ya = Y[:, ::-1, :]
    vr_ap, vt_ap, x_ap = sl_departure(vr, vt, x, E, dt, tau, vth, L, qe, me)
    ir, tr, ok_r = _cell(vrp, vr_ap)
    it, tt, ok_t = _cell(vta, vt_ap)
    ix, tx, ok_x = _cell(np.asarray(x), x_ap)
    out = np.zeros_like(vr_ap)
    for a in (0, 1):
        wa = tr if a else 1.0 - tr
        for b in (0, 1):
            wb = tt if b else 1.0 - tt
            for c in (0, 1):
                wc = tx if c else 1.0 - tx
                out += wa * wb * wc * Ya[ir + a, it + b, ix + c]
    out[~(ok_r & ok_t & ok_x)] = 0.0
    return out.reshape(Nr * Nvt, Nx)
