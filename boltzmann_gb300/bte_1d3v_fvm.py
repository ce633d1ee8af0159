"""The finite-volume 1D3V solver: its operator set-up and its steps on the GPU.

Counterpart of the reference's `bte_1d3v` with the FVM v-space (`vspace_type = 0`,
BESolver/python/bte_1d3v_solver.py): cells in v_r (the B-spline basis's per-interval Gauss
points) x discrete ordinates in theta x points in x, v laid out (Nr * Nvt, Nx), radial cell
major.

Set-up (host, once per dt; the reference builds the same on the host, :377-470,1333-1470):
* `radial_cells`: the v_r cells and their widths (spec_spherical.gl_vr with use_bspline_qgrid);
* `upwind_operator` / `upwind_operator_theta`: one-sided first-derivative operators
  (mesh.upwinded_dx / upwinded_dvt), weights by Fornberg's recursion;
* `FvmCollisions`: the strong-form electron-heavy operator
  (collision_operator_spherical.py:1334-1419) kept in its factored form
  C = G (x) (1 w^T) - diag(l) (x) I, G the (Nr x Nr) gain matrix, w = 2 pi (theta weights),
  l the loss rates. The collision inverse (I - c C)^-1 then has the closed form
  D^-1 (x) I + (c D^-1 G (D - c |w| G)^-1) (x) (1 w^T), D = I + c diag(l): an Nr x Nr solve,
  not the (Nr Nvt)^3 dense inverse (:1346-1375);
* `fvm_bands`: the six column-stored band arrays of the sweeps (:1403-1470).

Step (`FvmOpSplit`, :1745-1870, type XVTVRC) from the library's kernels
(`include/bte_sweeps_gb300.h`):
1. collisions: yc = PmatC v (bte_dgemm_nn);
2. v_r advection sweeps on (Nx, Nvt, Nr) (bte_adv_be_sweep kind 0, aE = tau qe / (me vth) E);
3. v_theta advection sweeps on (Nx, Nr, Nvt) (kind 1);
4. inflow zeroing and x advection sweeps on (Nr, Nvt, Nx) (kind 2, a = vth tau / L v_r cos theta).
The layout swaps between the stages run through bte_permute3.

Fully implicit step (`FvmImplicit`, `bte_1d3v_fvm.step`; :1890-2009) from the library's
`bte_fvm_*` entry points (`include/bte_fvm_gb300.h`): restarted GMRES on the fused operator
rhs_mvec, right-preconditioned with the op-split step, whose collision solve uses the
closed-form inverse instead of a dense PmatC. Semi-Lagrangian step (solver_type
"sl_implicit", :2024-2027,2244-2314): interpolation at the departure points, then the
closed-form collision inverse.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .bte_1d3v import (KB, ME, QE, chebyshev, load_params, ordinates, read_checkpoint, sph_ords_projections,
                       write_checkpoint)
from .native_kernels import _check, _ptr, _stream

C_GAMMA = math.sqrt(2.0 * QE / ME)   # v = C_GAMMA sqrt(eps [eV])


def thermal_velocity(Te_eV):
    """sqrt(2 k_B T / m_e) at T = Te_eV electron volts (collisions.py:20-25)."""
    return math.sqrt(2.0 * KB * (Te_eV * QE / KB) / ME)


# ----------------------------------------------------------------------------------
# grids
# ----------------------------------------------------------------------------------
def radial_cells(ev_max, Te, Nr, sp_order, spline_qpts):
    """The v_r cells (in units of vth): `spline_qpts` Gauss-Legendre points in each knot
    interval of the order-`sp_order` B-spline basis with Nr + 1 functions on uniform knots over
    [0, sqrt(ev_max) C_GAMMA / vth] (basis.py:414-429,640-653). Returns (vr, widths, vmax)."""
    vmax = math.sqrt(ev_max) * C_GAMMA / thermal_velocity(Te)
    n_int = Nr + 1 - sp_order
    if n_int < 1:
        raise ValueError("Nr + 1 must exceed sp_order")
    edges = np.linspace(0.0, vmax, n_int + 1)
    gx, gw = np.polynomial.legendre.leggauss(int(spline_qpts))
    half = 0.5 * np.diff(edges)
    mid = 0.5 * (edges[1:] + edges[:-1])
    vr = (half[:, None] * gx[None, :] + mid[:, None]).reshape(-1)
    qw = (half[:, None] * gw[None, :]).reshape(-1)
    return vr, qw, vmax


def x_points(Np, adaptive_grid=1):
    """x in [-1, 1] (bte_1d3v_solver.py:248-266, mesh.py:129-185; either x-space):
    Chebyshev-Gauss-Lobatto points when `adaptive_grid`, else uniform."""
    if adaptive_grid:
        return chebyshev(Np)[0]
    return np.linspace(-1.0, 1.0, Np)


# ----------------------------------------------------------------------------------
# upwind first derivatives
# ----------------------------------------------------------------------------------
def fd_weights(x0, nodes):
    """First-derivative weights at x0 on arbitrary nodes: the recursion of B. Fornberg,
    "Generation of finite difference formulas on arbitrarily spaced grids", Math. Comp. 51
    (1988) 699-706, carried to derivative order 1. Exact for polynomials of degree < len(nodes)."""
    z = np.asarray(nodes, dtype=np.float64)
    n = len(z)
    c = np.zeros((n, 2))
    c[0, 0] = 1.0
    prod_prev = 1.0
    dz_prev = z[0] - x0
    for i in range(1, n):
        prod = 1.0
        dz_i = z[i] - x0
        for j in range(i):
            d = z[i] - z[j]
            prod *= d
            if j == i - 1:
                c[i, 1] = prod_prev * (c[i - 1, 0] - dz_prev * c[i - 1, 1]) / prod
                c[i, 0] = -prod_prev * dz_prev * c[i - 1, 0] / prod
            c[j, 1] = (dz_i * c[j, 1] - c[j, 0]) / d
            c[j, 0] = dz_i * c[j, 0] / d
        prod_prev = prod
        dz_prev = dz_i
    return c[:, 1]


def upwind_operator(x, sw, direction):
    """Dense one-sided first-derivative operator on the points x (mesh.py:20-55): row i uses
    the up-to-sw points ending at i ("L") or starting at i ("R"); a row with a single point in
    its stencil (the first of "L", the last of "R") is zero."""
    x = np.asarray(x, dtype=np.float64)
    N = len(x)
    D = np.zeros((N, N))
    for i in range(N):
        lo, hi = (max(0, i - sw + 1), i + 1) if direction == "L" else (i, min(N, i + sw))
        if hi - lo > 1:
            D[i, lo:hi] = fd_weights(x[i], x[lo:hi])
    return D


def upwind_operator_theta(vt, sw, direction):
    """The ordinates' operator (mesh.py:80-112 without central differences): `upwind_operator`
    on each half of the ordinates, with the first row past the equator ("L", row N/2) or the
    last row before it ("R", row N/2 - 1) a two-point difference across it."""
    vt = np.asarray(vt, dtype=np.float64)
    N = len(vt)
    h = N // 2
    D = np.zeros((N, N))
    D[:h, :h] = upwind_operator(vt[:h], sw, direction)
    D[h:, h:] = upwind_operator(vt[h:], sw, direction)
    r = h if direction == "L" else h - 1
    D[r] = 0.0
    D[r, h - 1:h + 1] = fd_weights(vt[r], vt[h - 1:h + 1])
    return D


def band_columns(D, nd, lower):
    """The first nd diagonals of D stored the way the sweeps read them: lower
    band[k][i - k] = D[i][i - k], upper band[k][i + k] = D[i][i + k]."""
    N = D.shape[0]
    B = np.zeros((nd, N))
    for k in range(nd):
        if lower:
            B[k, :N - k] = np.diagonal(D, offset=-k)
        else:
            B[k, k:] = np.diagonal(D, offset=k)
    return B


def fvm_upwind_operators(vr, vt, x, pvr, pvt, px, vmax):
    """The dense upwind operators of the FVM solver with their boundary rows (:1406-1452,
    spec_spherical.py:909-926): inflow rows zero, the last v_r row of "R" the outflow
    -1 / (vmax - v_r[-1]), theta operators premultiplied by diag(sin theta)."""
    out = {"Dvr_L": upwind_operator(vr, pvr + 1, "L"), "Dvr_R": upwind_operator(vr, pvr + 1, "R"),
           "Dvt_L": upwind_operator_theta(vt, pvt + 1, "L"), "Dvt_R": upwind_operator_theta(vt, pvt + 1, "R"),
           "Dx_L": upwind_operator(x, px + 1, "L"), "Dx_R": upwind_operator(x, px + 1, "R")}
    for k in ("Dvr_L", "Dvt_L", "Dx_L"):
        out[k][0, :] = 0.0
    for k in ("Dvr_R", "Dvt_R", "Dx_R"):
        out[k][-1, :] = 0.0
    out["Dvr_R"][-1, -1] = -1.0 / (vmax - vr[-1])
    s = np.sin(np.asarray(vt))[:, None]
    out["Dvt_L"] = s * out["Dvt_L"]
    out["Dvt_R"] = s * out["Dvt_R"]
    return out


def fvm_bands(ops, pvr, pvt, px):
    """The sweeps' six band arrays (p + 1, N) from `fvm_upwind_operators` (:1452-1470)."""
    return dict(vr_diag_l2r=band_columns(ops["Dvr_L"], pvr + 1, True),
                vr_diag_r2l=band_columns(ops["Dvr_R"], pvr + 1, False),
                vt_diag_l2r=band_columns(ops["Dvt_L"], pvt + 1, True),
                vt_diag_r2l=band_columns(ops["Dvt_R"], pvt + 1, False),
                x_diag_l2r=band_columns(ops["Dx_L"], px + 1, True),
                x_diag_r2l=band_columns(ops["Dx_R"], px + 1, False))


# ----------------------------------------------------------------------------------
# collisions
# ----------------------------------------------------------------------------------
_KINDS = {"ELASTIC": 0, "EXCITATION": 1, "IONIZATION": 2}


def _sigma(proc, eps):
    """Tabulated total cross section, linear in energy, held at the end values outside the
    table (collisions.py:79)."""
    e = np.asarray(proc["energy"], dtype=np.float64)
    s = np.asarray(proc["cross section"], dtype=np.float64)
    return np.interp(eps, e, s, left=s[0], right=s[-1])


class FvmCollisions:
    """C = G (x) (1 w^T) - diag(loss) (x) I on the (v_r cell, ordinate) grid, index
    r * Nvt + j: gain G (Nr x Nr), loss (Nr), w = 2 pi theta weights (Nvt)."""

    def __init__(self, gain, loss, w):
        self.gain = np.asarray(gain, dtype=np.float64)
        self.loss = np.asarray(loss, dtype=np.float64)
        self.w = np.asarray(w, dtype=np.float64)
        self.Nr, self.Nvt = len(self.loss), len(self.w)

    def dense(self):
        return np.kron(self.gain, np.outer(np.ones(self.Nvt), self.w)) - np.kron(np.diag(self.loss), np.eye(self.Nvt))

    def apply(self, v):
        """C v for v (Nr * Nvt, ...) without forming C."""
        V = np.asarray(v).reshape((self.Nr, self.Nvt, -1))
        m = np.einsum("j,rjx->rx", self.w, V)
        out = (self.gain @ m)[:, None, :] - self.loss[:, None, None] * V
        return out.reshape(np.shape(v))

    def inverse_factors(self, c):
        """(dinv, H) with (I - c C)^-1 b = dinv (x) b + (H (x) 1) (w^T b): dinv = 1 / (1 + c loss),
        H = c D^-1 G (D - c |w| G)^-1."""
        d = 1.0 + c * self.loss
        A = np.diag(d) - (c * self.w.sum()) * self.gain
        H = (c / d)[:, None] * np.linalg.solve(A.T, self.gain.T).T
        return 1.0 / d, H

    def inverse_dense(self, c):
        """The dense (I - c C)^-1, the op-split step's PmatC."""
        dinv, H = self.inverse_factors(c)
        return np.kron(np.diag(dinv), np.eye(self.Nvt)) + np.kron(H, np.outer(np.ones(self.Nvt), self.w))


def fvm_collisions(processes, vr, vt_qw, vth, vmax):
    """The strong-form binary collision operator on the FVM grid
    (collision_operator_spherical.py:1334-1419), summed over `processes` (the
    `read_cross_section_data` dicts; each needs "type", "threshold", "energy", "cross section",
    and the elastic ones "mass_ratio"). Per process, with s(v) = v vth sigma(eps(v)) / (4 pi):
    loss 4 pi s(v_r); gain s(v_pre) J times f at v_pre, linearly interpolated between cells,
    zero below the first cell and falling linearly to 0 at vmax past the last, averaged over
    theta. v_pre, J: elastic v / sqrt(1 - 2 m/M), (1 - 2 m/M)^(-3/2); excitation
    sqrt(v^2 + (C_GAMMA/vth)^2 eps_th), v_pre / v; ionization sqrt(2 v^2 + (C_GAMMA/vth)^2
    eps_th), 4 v_pre / v."""
    vr = np.asarray(vr, dtype=np.float64)
    Nr = len(vr)
    gain = np.zeros((Nr, Nr))
    loss = np.zeros(Nr)
    k2 = (C_GAMMA / vth) ** 2
    for proc in processes:
        kind = str(proc["type"]).upper()
        if kind not in _KINDS:
            raise NotImplementedError("no strong-form FVM operator for %s processes" % kind)
        if _KINDS[kind] == 0:
            scale = math.sqrt(1.0 - 2.0 * float(proc["mass_ratio"]))
            vpre = vr / scale
            J = np.full(Nr, scale ** -3)
        elif _KINDS[kind] == 1:
            vpre = np.sqrt(vr ** 2 + k2 * float(proc["threshold"]))
            J = vpre / vr
        else:
            vpre = np.sqrt(2.0 * vr ** 2 + k2 * float(proc["threshold"]))
            J = 4.0 * vpre / vr
        s = vr * vth * _sigma(proc, (vr * vth / C_GAMMA) ** 2) / (4.0 * math.pi)
        s_pre = vpre * vth * _sigma(proc, (vpre * vth / C_GAMMA) ** 2) / (4.0 * math.pi)
        # linear interpolation weights of the cell values at v_pre
        k = np.clip(np.searchsorted(vr, vpre, side="right") - 1, 0, Nr - 2)
        t = (vpre - vr[k]) / (vr[k + 1] - vr[k])
        inside = (vpre >= vr[0]) & (vpre <= vr[-1])
        tail = (vpre > vr[-1]) & (vpre <= vmax)
        rows = np.arange(Nr)
        W = np.zeros((Nr, Nr))
        W[rows[inside], k[inside]] += 1.0 - t[inside]
        W[rows[inside], k[inside] + 1] += t[inside]
        W[rows[tail], Nr - 1] = (vmax - vpre[tail]) / (vmax - vr[-1])
        gain += (s_pre * J)[:, None] * W
        loss += 4.0 * math.pi * s
    return gain, loss


# ----------------------------------------------------------------------------------
# quantities of interest
# ----------------------------------------------------------------------------------
TEMP_K_1EV = QE / KB


def fvm_qoi_functionals(processes, vr, vr_qw, vt_qw, vth):
    """The FVM grid's QoI functionals (bte_1d3v_solver.py:493-502), rows of a (2 + n_proc) x
    (Nr * Nvt) matrix: mass 2 pi (v_r^2 dv_r (x) w_theta); temperature in eV
    2 pi vth^2 (v_r^4 dv_r (x) w_theta) 0.5 me (2 / 3 / kB) / (e / kB); per process the rate
    2 pi (2 vth^4 / c_gamma^3) (v_r^3 dv_r sigma(eps(v_r)) (x) w_theta)."""
    vr, vr_qw, vt_qw = (np.asarray(a, dtype=np.float64) for a in (vr, vr_qw, vt_qw))
    ev_fac = 0.5 * ME * (2.0 / 3.0 / KB) / TEMP_K_1EV
    rows = [2.0 * np.pi * np.kron(vr ** 2 * vr_qw, vt_qw),
            2.0 * np.pi * vth ** 2 * np.kron(vr ** 4 * vr_qw, vt_qw) * ev_fac]
    for proc in processes:
        sig = _sigma(proc, (vr * vth / C_GAMMA) ** 2)
        rows.append(2.0 * np.pi * (2.0 * vth ** 4 / C_GAMMA ** 3) * np.kron(vr ** 3 * vr_qw * sig, vt_qw))
    return np.array(rows)


def qoi_from_moments(Y, vth, np0, mass_scale):
    """compute_qoi (bte_1d3v_solver.py:1179-1215) from Y = Q v, Q the (2 + n_proc) QoI rows:
    ne = m0 np0, Te = (temp . v) / m0, rates = (rate . v) / s with the normalization
    s = m0 / mass_scale * 2 (vth / c_gamma)^3 (mass_scale 1 on the FVM grid, sqrt(4 pi) for the
    harmonics); mobility and diffusion are 0, as the reference returns. Works on NumPy arrays
    and on tensors; rates are (Nx, n_proc)."""
    m0 = Y[0]
    scale = m0 / mass_scale * (2.0 * (vth / C_GAMMA) ** 3)
    return {"rates": (Y[2:] / scale).T, "mu": 0.0, "D": 0.0, "ne": m0 * np0, "Te": Y[1] / m0}


def fvm_radial_components(vsh, vr, nsh, ev, vth):
    """compute_radial_components on the FVM grid (bte_1d3v_solver.py:1162-1177): the harmonics
    vsh (Nr * nsh, Nx) interpolated linearly in v_r at v(eps) = sqrt(eps) c_gamma / vth;
    returns (Nx, nsh, len(ev)). An energy whose speed lies outside the cells raises ValueError,
    as the reference's interpolation (bounds_error=True) does."""
    vr = np.asarray(vr, dtype=np.float64)
    Nr = len(vr)
    V = np.asarray(vsh, dtype=np.float64).reshape(Nr, nsh, -1)
    q = np.sqrt(np.asarray(ev, dtype=np.float64)) * C_GAMMA / vth
    if np.any(q < vr[0]) or np.any(q > vr[-1]):
        raise ValueError("an energy's speed lies outside the cells [%.6g, %.6g]" % (vr[0], vr[-1]))
    i = np.clip(np.searchsorted(vr, q, side="right") - 1, 0, Nr - 2)
    t = (q - vr[i]) / (vr[i + 1] - vr[i])
    lo = V[i].transpose(2, 1, 0)       # (Nx, nsh, n_ev)
    hi = V[i + 1].transpose(2, 1, 0)
    return (1.0 - t) * lo + t * hi


# ----------------------------------------------------------------------------------
# the op-split step on the GPU
# ----------------------------------------------------------------------------------
class FvmOpSplit:
    """PmatC (dof_v x dof_v), band arrays (p+1, N) of the three directions, grids vr (Nr),
    vt (Nvt), and the coefficients tau, qe, me, vth, L of the reference's parameters."""

    def __init__(self, PmatC, vr_diag_l2r, vr_diag_r2l, vt_diag_l2r, vt_diag_r2l, x_diag_l2r, x_diag_r2l, vr, vt,
                 Nx, tau, qe, me, vth, L, device=None):
        import torch
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
        self.Nr, self.Nvt, self.Nx = len(vr), len(vt), int(Nx)
        if np.shape(PmatC) != (self.Nr * self.Nvt, self.Nr * self.Nvt):
            raise ValueError("PmatC must be (Nr * Nvt) x (Nr * Nvt)")
        self.P = t(PmatC)
        self.bands = [(t(vr_diag_l2r), t(vr_diag_r2l)), (t(vt_diag_l2r), t(vt_diag_r2l)), (t(x_diag_l2r), t(x_diag_r2l))]
        for (l, r), n in zip(self.bands, (self.Nr, self.Nvt, self.Nx)):
            if l.shape[1] != n or r.shape[1] != n or l.shape[0] != r.shape[0]:
                raise ValueError("band arrays must be (p + 1, N) for their direction")
        self.vr, self.vt = t(vr), t(vt)
        self.cos_vt = t(np.cos(np.asarray(vt)))
        self.cE = float(tau) * float(qe) / float(me) / float(vth)
        self.ax = float(vth) * (float(tau) / float(L))
        self.ax_vr = t(self.ax * np.asarray(vr))
        n = self.Nr * self.Nvt * self.Nx
        self._a = torch.empty(n, dtype=torch.float64, device=dev)
        self._b = torch.empty(n, dtype=torch.float64, device=dev)
        self.dev = dev

    def step(self, E, v, dt, alpha=1.0):
        """One op-split step: v (Nr * Nvt, Nx) CUDA float64, E (Nx) the field -> new v."""
        import torch
        lib, s = _lib.load(), _stream()
        Nr, Nvt, Nx = self.Nr, self.Nvt, self.Nx
        dof = Nr * Nvt
        v = v.contiguous()
        if v.numel() != dof * Nx or not v.is_cuda or v.dtype != torch.float64:
            raise ValueError("v must be a (Nr * Nvt, Nx) float64 CUDA tensor")
        aE = torch.as_tensor(np.asarray(E), dtype=torch.float64, device=self.dev) * self.cE
        if aE.numel() != Nx:
            raise ValueError("E must have Nx values")
        h = float(alpha) * float(dt)
        a, b = self._a, self._b
        _check(lib.bte_dgemm_nn(dof, Nx, dof, _ptr(self.P), dof, _ptr(v), Nx, _ptr(a), Nx, s), "collision solve")
        # (Nr, Nvt, Nx) -> (Nx, Nvt, Nr)
        _check(lib.bte_permute3(Nr, Nvt, Nx, 2, 1, 0, _ptr(a), _ptr(b), s), "layout")
        (l, r) = self.bands[0]
        _check(lib.bte_adv_be_sweep(0, _ptr(l), _ptr(r), _ptr(aE), _ptr(self.cos_vt), h, _ptr(b), _ptr(a), l.shape[0],
                                    Nr, Nvt, Nx, s), "v_r sweep")
        # (Nx, Nvt, Nr) -> (Nx, Nr, Nvt)
        _check(lib.bte_permute3(Nx, Nvt, Nr, 0, 2, 1, _ptr(a), _ptr(b), s), "layout")
        (l, r) = self.bands[1]
        _check(lib.bte_adv_be_sweep(1, _ptr(l), _ptr(r), _ptr(aE), _ptr(self.vr), h, _ptr(b), _ptr(a), l.shape[0],
                                    Nr, Nvt, Nx, s), "v_theta sweep")
        # (Nx, Nr, Nvt) -> (Nr, Nvt, Nx)
        _check(lib.bte_permute3(Nx, Nr, Nvt, 1, 2, 0, _ptr(a), _ptr(b), s), "layout")
        _check(lib.bte_fvm_inflow_zero(Nr, Nvt, Nx, _ptr(self.vt), _ptr(b), s), "inflow")
        (l, r) = self.bands[2]
        out = torch.empty(dof, Nx, dtype=torch.float64, device=self.dev)
        _check(lib.bte_adv_be_sweep(2, _ptr(l), _ptr(r), _ptr(self.ax_vr), _ptr(self.cos_vt), h, _ptr(b), _ptr(out),
                                    l.shape[0], Nr, Nvt, Nx, s), "x sweep")
        return out


# ----------------------------------------------------------------------------------
# the fully implicit step on the GPU
# ----------------------------------------------------------------------------------
_BAND_KEYS = ("vr_diag_l2r", "vr_diag_r2l", "vt_diag_l2r", "vt_diag_r2l", "x_diag_l2r", "x_diag_r2l")


def _host(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class FvmImplicit:
    """The library's fully implicit FVM step (include/bte_fvm_gb300.h) on one GPU: the fused
    operator (rhs_mvec), the op-split preconditioner with the closed-form collision inverse,
    and the GMRES solve. Set-up: grids vr (Nr), vt (Nvt), the ordinate weights vt_qw, Nx,
    `bands` (the six arrays of `fvm_bands`) and `coll` (an `FvmCollisions`)."""

    def __init__(self, vr, vt, vt_qw, Nx, bands, coll, device=0):
        import torch
        self.torch = torch
        self.device = int(device)
        self.Nr, self.Nvt, self.Nx = len(vr), len(vt), int(Nx)
        b = [_host(bands[k]) for k in _BAND_KEYS]
        for (l, r), n in zip(((b[0], b[1]), (b[2], b[3]), (b[4], b[5])), (self.Nr, self.Nvt, self.Nx)):
            if l.ndim != 2 or l.shape != r.shape or l.shape[1] != n:
                raise ValueError("band arrays must be (p + 1, N) for their direction")
        if coll.Nr != self.Nr or coll.Nvt != self.Nvt:
            raise ValueError("collision operator and grids disagree in size")
        self.coll = coll
        self._keep = [_host(vr), _host(vt), _host(2.0 * np.pi * np.asarray(vt_qw)), _host(coll.loss), _host(coll.gain)] + b
        h = C.c_void_p()
        lib = _lib.load()
        rc = lib.bte_fvm_create(self.device, self.Nr, self.Nvt, self.Nx, b[0].shape[0], b[2].shape[0], b[4].shape[0],
                                *[_dp(a) for a in self._keep], C.byref(h))
        self._fail(rc, "bte_fvm_create")
        self._h = h
        self.gmres_info = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._h = None
            try:
                _lib.load().bte_fvm_destroy(h)
            except Exception:   # interpreter shutdown: the library may already be gone
                pass

    @staticmethod
    def _fail(rc, what):
        if rc != 0:
            raise RuntimeError("%s failed (%d): %s" % (what, rc, _lib.load().bte_fvm_last_error().decode()))

    def _dev(self, a, n):
        t = self.torch.as_tensor(a, dtype=self.torch.float64, device="cuda")
        if t.numel() != n:
            raise ValueError("expected %d values, got %d" % (n, t.numel()))
        return t.reshape(-1).contiguous()

    def set_collision_inverse(self, c):
        """Preconditioner collision solve (I - c C)^-1, c = gmres_pc_cv dt tau n0 np0."""
        dinv, H = self.coll.inverse_factors(float(c))
        self._inv = (_host(dinv), _host(H))
        self._fail(_lib.load().bte_fvm_set_collision_inverse(self._h, _dp(self._inv[0]), _dp(self._inv[1])),
                   "bte_fvm_set_collision_inverse")

    def mvec(self, coef, E, X):
        """rhs_mvec(X) with coef an `_lib.FvmCoef`; X (Nr * Nvt, Nx) -> CUDA tensor of its shape."""
        n = self.Nr * self.Nvt * self.Nx
        Xd, Ed = self._dev(X, n), self._dev(E, self.Nx)
        Y = self.torch.empty_like(Xd)
        self._fail(_lib.load().bte_fvm_mvec(self._h, C.byref(coef), _ptr(Ed), _ptr(Xd), _ptr(Y), _stream()),
                   "bte_fvm_mvec")
        return Y.reshape(self.Nr * self.Nvt, self.Nx)

    def precond(self, cE, ax, hstep, E, X):
        """The op-split step (XVTVRC) of X at aE = cE E, x coefficient ax, step hstep."""
        n = self.Nr * self.Nvt * self.Nx
        Xd, Ed = self._dev(X, n), self._dev(E, self.Nx)
        Y = self.torch.empty_like(Xd)
        self._fail(_lib.load().bte_fvm_precond(self._h, float(cE), float(ax), float(hstep), _ptr(Ed), _ptr(Xd),
                                               _ptr(Y), _stream()), "bte_fvm_precond")
        return Y.reshape(self.Nr * self.Nvt, self.Nx)

    def step(self, coef, E, V, alpha=1.0, rtol=1e-12, atol=1e-14, restart=30, max_iter=600, pc_mode=0):
        """Solve rhs_mvec(V') = V (inflow values zeroed); pc_mode 0: the op-split preconditioner
        on the right, 1: on the left, 2: none. Returns V' (Nr * Nvt, Nx)."""
        n = self.Nr * self.Nvt * self.Nx
        Vd, Ed = self._dev(V, n).clone(), self._dev(E, self.Nx)
        info = (C.c_double * 4)()
        rc = _lib.load().bte_fvm_step(self._h, C.byref(coef), float(alpha), int(pc_mode), _ptr(Ed), _ptr(Vd),
                                      float(rtol), float(atol), int(restart), int(max_iter), info, _stream())
        self._fail(rc, "bte_fvm_step")
        self.gmres_info = {"iterations": int(info[0]), "residual_abs": info[1], "residual_rel": info[2],
                           "status": int(info[3])}
        return Vd.reshape(self.Nr * self.Nvt, self.Nx)

    def set_sl_grid(self, x, vmin, vmax):
        """Grids of the semi-Lagrangian step: the x points and the cells' velocity domain."""
        self._xg = _host(x)
        if len(self._xg) != self.Nx:
            raise ValueError("x must have Nx points")
        self._fail(_lib.load().bte_fvm_set_sl_grid(self._h, _dp(self._xg), float(vmin), float(vmax)),
                   "bte_fvm_set_sl_grid")

    def sl_advect(self, coef, E, V):
        """step_adv_vx_sl: V interpolated at its departure points over coef.dt."""
        n = self.Nr * self.Nvt * self.Nx
        Vd, Ed = self._dev(V, n), self._dev(E, self.Nx)
        Y = self.torch.empty_like(Vd)
        self._fail(_lib.load().bte_fvm_sl_advect(self._h, C.byref(coef), _ptr(Ed), _ptr(Vd), _ptr(Y), _stream()),
                   "bte_fvm_sl_advect")
        return Y.reshape(self.Nr * self.Nvt, self.Nx)

    def sl_step(self, coef, E, V):
        """One semi-Lagrangian step: the collision inverse of sl_advect(V)."""
        n = self.Nr * self.Nvt * self.Nx
        Vd, Ed = self._dev(V, n), self._dev(E, self.Nx)
        Y = self.torch.empty_like(Vd)
        self._fail(_lib.load().bte_fvm_sl_step(self._h, C.byref(coef), _ptr(Ed), _ptr(Vd), _ptr(Y), _stream()),
                   "bte_fvm_sl_step")
        return Y.reshape(self.Nr * self.Nvt, self.Nx)

    def launches(self):
        return int(_lib.load().bte_fvm_launches(self._h))


# ----------------------------------------------------------------------------------
# the reference-facing solver
# ----------------------------------------------------------------------------------
XVTVRC = 3          # pc_type.XVTVRC (bte_1d3v_solver.py:58-63), the one op-split order the reference implements
_SOLVERS = {"fully_implicit": "fully_implicit", "XVTVRC": "op_split", "sl_implicit": "semi_lagrangian"}


def fvm_setup(par):
    """The host set-up of the FVM solver from the reference's parameter table (a TOML path with a
    [bte] table, or the table as a dict): vspace_type = 0, solver_type "fully_implicit" or
    "XVTVRC" or "sl_implicit", pc_type "xvtvrc_solve" (the default) or "none", `collisions` an
    LXCat file. Returns a
    namespace: params, vth, vmax, vr, vr_qw, vt, vt_qw, x, grid_info, collisions (an
    `FvmCollisions`), bands (the six `fvm_bands` arrays). Mirrors bte_1d3v.__init__ / init()
    (bte_1d3v_solver.py:77-216,245-266,377-470,1403-1470)."""
    import types
    from .lxcat import read_cross_section_data
    tp = par
    if not isinstance(par, dict):
        import tomllib
        with open(par, "rb") as fh:
            tp = tomllib.load(fh)["bte"]
    p = load_params(tp, fvm=True)
    p.pvr, p.pvt, p.px = int(tp.get("pvr", 3)), int(tp.get("pvt", 3)), int(tp.get("px", 1))
    p.adaptive_grid = bool(tp.get("adaptive_grid", 1))
    p.pc_type = str(tp.get("pc_type", "xvtvrc_solve"))
    if p.pc_type not in ("xvtvrc_solve", "none"):
        raise NotImplementedError("pc_type must be the op-split XVTVRC preconditioner or none")
    if tp.get("solver_type") not in _SOLVERS:
        raise NotImplementedError("solver_type must be one of %s for the FVM v-space" % sorted(_SOLVERS))
    p.solver = _SOLVERS[tp["solver_type"]]
    if p.solver == "fully_implicit" and int(tp.get("xspace_type", 1)) != 0:
        # the reference's rhs_mvec needs the banded x-shift, which it builds only for the upwind
        # x-space (bte_1d3v_solver.py:843-861, 1938-1939)
        raise NotImplementedError("the fully implicit FVM step needs xspace_type = 0 (upwind x)")
    if tp.get("ic_file", ""):
        raise NotImplementedError("initial conditions from files are not provided")
    p.qe, p.me = QE, ME
    vth = thermal_velocity(p.Te)
    vr, vr_qw, vmax = radial_cells(p.ev_max, p.Te, p.Nr, p.sp_order, p.spline_qpts)
    vt, vt_qw = ordinates(p.Nvt)
    x = x_points(p.Np, p.adaptive_grid)
    procs = list(read_cross_section_data(p.collisions).values())
    gain, loss = fvm_collisions(procs, vr, vt_qw, vth, vmax)
    coll = FvmCollisions(gain, loss, 2.0 * np.pi * vt_qw)
    bands = fvm_bands(fvm_upwind_operators(vr, vt, x, p.pvr, p.pvt, p.px, vmax), p.pvr, p.pvt, p.px)
    return types.SimpleNamespace(params=p, vth=vth, vmax=vmax, vr=vr, vr_qw=vr_qw, vt=vt, vt_qw=vt_qw, x=x,
                                 grid_info={"x": x, "vr": vr, "vr_qw": vr_qw, "vt": vt, "vt_qw": vt_qw},
                                 collisions=coll, bands=bands,
                                 qoi=fvm_qoi_functionals(procs, vr, vr_qw, vt_qw, vth))


def fvm_initial_condition(p, vth, vr, Nvt, x):
    """initial_condition(type=0) for the FVM v-space (bte_1d3v_solver.py:1288-1327): the density
    profile ne(x) times a Maxwellian at Te in every cell and ordinate; (Nr * Nvt, Nx)."""
    xx = p.L * (np.asarray(x) + 1)
    ne = 1e6 * (1e7 + 1e9 * (1 - 0.5 * xx / p.L) ** 2 * (0.5 * xx / p.L) ** 2) / p.np0
    ratio = C_GAMMA * math.sqrt(p.Te) / vth
    hv = np.exp(-(np.asarray(vr) / ratio) ** 2) / (math.sqrt(math.pi) ** 3 * ratio ** 3)
    return np.kron(hv, np.ones(Nvt))[:, None] * ne[None, :]


def step_coefficients(p, vth, dt, dtx):
    """(dt, dtx, tau, kappa, cA, ax) of a step (bte_fvm_coef): kappa = n0 np0, cA = qe / (me vth),
    ax = vth tau / L (bte_1d3v_solver.py:1775-1776); dtx the x-shift's set-up step."""
    return (float(dt), float(dtx), p.tau, p.n0 * p.np0, QE / ME / vth, vth * (p.tau / p.L))


class bte_1d3v_fvm:
    """The reference's `bte_1d3v` with the finite-volume v-space on one GPU. `par`: the
    parameter file (TOML with a [bte] table) or the same table as a dict, with
    vspace_type = 0 and solver_type "fully_implicit", "XVTVRC" or "sl_implicit"; `collisions`
    names an LXCat file (single species)."""

    def __init__(self, par, device=0):
        import torch
        self.torch = torch
        st = fvm_setup(par)
        self.params = p = st.params
        self.device = int(device)
        torch.cuda.set_device(self.device)
        self.bs_vth, self.vmax, self.xp = st.vth, st.vmax, st.x
        self.grid_info = st.grid_info
        self.dof_vr, self.dof_vt, self.dof_x = len(st.vr), len(st.vt), p.Np
        self.dof_v = self.dof_vr * self.dof_vt
        self.op_col, self.bands = st.collisions, st.bands
        self.op_qoi = torch.as_tensor(st.qoi, dtype=torch.float64, device="cuda")
        self.num_sh = p.l_max + 1
        psh2o, po2sh = sph_ords_projections(st.vt, st.vt_qw, p.l_max)
        self.op_psh2o = torch.as_tensor(psh2o, dtype=torch.float64, device="cuda").contiguous()
        self.op_po2sh = torch.as_tensor(po2sh, dtype=torch.float64, device="cuda").contiguous()
        self.solver = FvmImplicit(st.vr, st.vt, st.vt_qw, p.Np, self.bands, self.op_col, device=self.device)
        self.solver.set_sl_grid(st.x, 0.0, self.vmax)
        self.c_gamma = C_GAMMA
        self.gmres_info = None
        self._dt_init = None

    def init(self, dt, gmres_pc_cv=1.0, gmres_pc_ax=1.0):
        """init(dt) (:1333-1470): the collision inverse at gmres_pc_cv dt and the x-shift at
        gmres_pc_ax dt."""
        p = self.params
        self.solver.set_collision_inverse(gmres_pc_cv * dt * p.tau * p.n0 * p.np0)
        self._dt_init = gmres_pc_ax * dt

    def _coef(self, dt):
        from ._lib import FvmCoef
        if self._dt_init is None:
            raise RuntimeError("init(dt) must be called before stepping")
        return FvmCoef(*step_coefficients(self.params, self.bs_vth, dt, self._dt_init))

    def rhs_mvec(self, E, x, dt):
        """The fully implicit step's operator applied to x (Nr * Nvt, Nx) (:1915-1955)."""
        return self.solver.mvec(self._coef(dt), E, x)

    def step_op_split(self, E, v, dv, time, dt, type=XVTVRC, verbose=0, alpha=1.0):
        """step_op_split (:1745-1870), type XVTVRC: returns the new (Nr * Nvt, Nx) state."""
        if type != XVTVRC:
            raise NotImplementedError("preconditioner type not implemented")
        c = self._coef(dt)
        return self.solver.precond(c.tau * c.cA, c.ax, float(alpha) * float(dt), E, v)

    def step_adv_vx_sl(self, E, v, time, dt, verbose=0):
        """step_adv_vx_sl (:2244-2314): v interpolated at its departure points over dt."""
        return self.solver.sl_advect(self._coef(dt), E, v)

    def step(self, E, v, dv, time, dt, verbose=0, gmres_pc_vr=1.0, gmres_pc_vt=1.0, pc_left=False):
        """step (:1872-2030): the fully implicit solve (GMRES preconditioned by the op-split
        step at gmres_pc_vr dt, on the left when pc_left); with solver_type "XVTVRC" one op-split
        step; with "sl_implicit" the collision inverse of the semi-Lagrangian advection
        (:2024-2027)."""
        p = self.params
        if p.solver == "op_split":
            return self.step_op_split(E, v, dv, time, dt, XVTVRC, verbose)
        if p.solver == "semi_lagrangian":
            return self.solver.sl_step(self._coef(dt), E, v)
        mode = 2 if p.pc_type == "none" else (1 if pc_left else 0)
        out = self.solver.step(self._coef(dt), E, v, alpha=gmres_pc_vr, rtol=p.rtol, atol=p.atol,
                               restart=p.gmres_rsrt, max_iter=p.gmres_maxiter, pc_mode=mode)
        info = self.solver.gmres_info
        self.gmres_info = info
        if info["status"] != 0:
            raise RuntimeError("%08d GMRES solver failed! iterations =%d  ||res|| = %.4E ||res||/||b|| = %.4E"
                               % (int(time / dt), info["iterations"], info["residual_abs"], info["residual_rel"]))
        return out

    def initial_condition(self, type=0):
        """initial_condition(type=0) (:1288-1327), on the device."""
        if type != 0:
            raise NotImplementedError
        v = fvm_initial_condition(self.params, self.bs_vth, self.grid_info["vr"], self.dof_vt, self.xp)
        return self.torch.as_tensor(v, dtype=self.torch.float64, device="cuda")

    def _project(self, P, x, n_in, n_out):
        """(Nr, n_in, Nx) -> (Nr, n_out, Nx) by P (n_out x n_in) along the middle axis: two layout
        swaps (bte_permute3) around one FP64 GEMM (bte_dgemm_nn)."""
        torch = self.torch
        lib, s = _lib.load(), _stream()
        Nr, Nx = self.dof_vr, self.dof_x
        X = torch.as_tensor(x, dtype=torch.float64, device="cuda").reshape(-1).contiguous()
        if X.numel() != Nr * n_in * Nx:
            raise ValueError("expected (%d, %d) values" % (Nr * n_in, Nx))
        A = torch.empty(Nr * n_in * Nx, dtype=torch.float64, device="cuda")
        B = torch.empty(Nr * n_out * Nx, dtype=torch.float64, device="cuda")
        _check(lib.bte_permute3(Nr, n_in, Nx, 1, 0, 2, _ptr(X), _ptr(A), s), "layout")        # (n_in, Nr, Nx)
        _check(lib.bte_dgemm_nn(n_out, Nr * Nx, n_in, _ptr(P), n_in, _ptr(A), Nr * Nx, _ptr(B), Nr * Nx, s),
               "projection")
        out = torch.empty(Nr * n_out * Nx, dtype=torch.float64, device="cuda")
        _check(lib.bte_permute3(n_out, Nr, Nx, 1, 0, 2, _ptr(B), _ptr(out), s), "layout")     # (Nr, n_out, Nx)
        return out.reshape(Nr * n_out, Nx)

    def ords_to_sph(self, x):
        """ords_to_sph (:678-685): (Nr * Nvt, Nx) ordinates -> (Nr * num_sh, Nx) harmonics."""
        return self._project(self.op_po2sh, x, self.dof_vt, self.num_sh)

    def sph_to_ords(self, x):
        """sph_to_ords (:687-694): (Nr * num_sh, Nx) harmonics -> (Nr * Nvt, Nx) ordinates."""
        return self._project(self.op_psh2o, x, self.num_sh, self.dof_vt)

    def store_checkpoint(self, v, time, dt, fprefix):
        """store_checkpoint (:2065-2090): v with its ne and Te, to `fprefix`.npz."""
        q = self.compute_qoi(v, time, dt)
        write_checkpoint(fprefix, v, time, dt, q["ne"], q["Te"])

    def restore_checkpoint(self, fprefix):
        """restore_checkpoint (:2092-2103): (time, dt, v) with v on the device."""
        t, dt, v = read_checkpoint(fprefix)
        return t, dt, self.torch.as_tensor(v, dtype=self.torch.float64, device="cuda")

    def normalize_edf(self, v):
        """normalize_edf (:2043-2062) on the FVM grid: v / ((mass . v) 2 (vth / c_gamma)^3) per x."""
        V = self.torch.as_tensor(v, dtype=self.torch.float64, device="cuda").reshape(self.dof_v, self.dof_x)
        return V / ((self.op_qoi[0] @ V) * (2.0 * (self.bs_vth / C_GAMMA) ** 3))

    def asnumpy(self, x):
        return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)

    def copy_operators_H2D(self, dev_id=0):
        """The operators live on the device from construction on: nothing to copy."""

    def copy_operators_D2H(self, dev_id=0):
        """The operators stay on the device; host copies are the set-up's (fvm_setup)."""

    def compute_radial_components(self, ev, v):
        """compute_radial_components (:1162-1177): (Nx, num_sh, len(ev)) NumPy array."""
        vsh = self.ords_to_sph(v).cpu().numpy()
        return fvm_radial_components(vsh, self.grid_info["vr"], self.num_sh, ev, self.bs_vth)

    def compute_qoi(self, v, time, dt):
        """compute_qoi (:1179-1215) per x point: "rates" (Nx, n_proc), "ne", "Te"; "mu" and "D"
        are 0 as in the reference. The QoI rows multiply v in one FP64 GEMM (bte_dgemm_nn)."""
        torch = self.torch
        V = torch.as_tensor(v, dtype=torch.float64, device="cuda").reshape(self.dof_v, self.dof_x).contiguous()
        Q = self.op_qoi
        Y = torch.empty((Q.shape[0], self.dof_x), dtype=torch.float64, device="cuda")
        _check(_lib.load().bte_dgemm_nn(Q.shape[0], self.dof_x, self.dof_v, _ptr(Q), self.dof_v, _ptr(V), self.dof_x,
                                        _ptr(Y), self.dof_x, _stream()), "QoI functionals")
        return qoi_from_moments(Y, self.bs_vth, self.params.np0, 1.0)

    def launches(self):
        return self.solver.launches()
