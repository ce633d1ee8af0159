// Shared host/device core of the finite-volume 1D3V fully implicit step: the per-element
// arithmetic of its operator and preconditioner, and its restarted GMRES. The CUDA kernels in
// fvm.cu wrap these functions one thread per element; the same code compiles for the host, so
// the arithmetic and the solver loop are checked against the oracle without a GPU.
//
// State v (double) is the reference's (Nr * Nvt, Nx) array: v[(r * Nvt + j) * Nx + x], r the
// radial cell, j the ordinate, x the spatial point.
//
// Operator (rhs_mvec, bte_1d3v_solver.py:1915-1955):
//   y = X v - dt tau (kappa C v + E (x) cA A_sign(E) v), the second term zero on inflow rows,
//   X v = v + dtx ax v_r cos(theta_j) Dx v   (x-shift, :780-860; Dx upwind "L" for theta <= pi/2)
//   C v = G (w^T v) - loss (x) v            (factored collision operator)
//   A_Ep v = cos(theta_j) Dvr_(R if cos > 0 else L) v - (1/v_r) sinDvt_R v, A_En with L and R
//   swapped (spec_spherical.py:876-951).
// All upwind operators are the sweeps' column-stored bands: lower D[i][i-k] = B[k][i-k], upper
// D[i][i+k] = B[k][i+k].
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#if defined(__CUDACC__)
#define FVM_HD __host__ __device__ inline
#else
#define FVM_HD inline
#endif

struct FvmView {
    int Nr, Nvt, Nx;
    int ndr, ndt, ndx;            // stored diagonals of the v_r, v_theta and x bands
    const double* vr;             // Nr cell centres, units of vth
    const double* cos_t;          // Nvt
    const int8_t* north;          // Nvt: 1 when theta_j <= pi/2 (inflow at the first x point)
    const double* w;              // Nvt: 2 pi times the ordinate weights
    const double* loss;           // Nr: collision loss rates
    const double *vrL, *vrR;      // (ndr, Nr)
    const double *vtL, *vtR;      // (ndt, Nvt), sin(theta)-scaled
    const double *xL, *xR;        // (ndx, Nx)
};

// dt: the step; dtx: the step the x-shift is set up with; kappa = n0 np0; cA = qe / (me vth);
// ax = vth tau / L
struct FvmCoef {
    double dt, dtx, tau, kappa, cA, ax;
};

// sum_k D[i][i -/+ k] z[(i -/+ k) stride] for a column-stored band over a line of N values
FVM_HD double fvm_band_row(const double* B, int nd, int N, int i, bool lower, const double* z, long long stride) {
    double s = 0.0;
    if (lower) {
        for (int k = 0; k < nd && k <= i; ++k) s += B[(size_t)k * N + (i - k)] * z[(long long)(i - k) * stride];
    } else {
        for (int k = 0; k < nd && i + k < N; ++k) s += B[(size_t)k * N + (i + k)] * z[(long long)(i + k) * stride];
    }
    return s;
}

FVM_HD bool fvm_inflow(const FvmView& v, int j, int x) { return v.north[j] ? x == 0 : x == v.Nx - 1; }

// the ordinate moment m[r][x] = sum_j w_j v[r][j][x]
FVM_HD double fvm_moment_at(const FvmView& v, const double* X, int r, int x) {
    const double* p = X + (size_t)r * v.Nvt * v.Nx + x;
    double s = 0.0;
    for (int j = 0; j < v.Nvt; ++j) s += v.w[j] * p[(size_t)j * v.Nx];
    return s;
}

// rhs_mvec at (r, j, x); G = gain (Nr x Nr) applied to the moments of X, (Nr, Nx)
FVM_HD double fvm_mvec_at(const FvmView& v, const FvmCoef& c, const double* E, const double* G, const double* X, int r,
                          int j, int x) {
    const size_t line = ((size_t)r * v.Nvt + j) * v.Nx;
    const double z = X[line + x];
    const bool nx = v.north[j] != 0;
    const double dx = fvm_band_row(nx ? v.xL : v.xR, v.ndx, v.Nx, x, nx, X + line, 1);
    const double yx = z + c.dtx * c.ax * v.vr[r] * v.cos_t[j] * dx;
    if (fvm_inflow(v, j, x)) return yx;
    const double e = E[x];
    const bool up_r = (e >= 0.0) == (v.cos_t[j] > 0.0);
    const double dr = fvm_band_row(up_r ? v.vrR : v.vrL, v.ndr, v.Nr, r, !up_r, X + (size_t)j * v.Nx + x,
                                   (long long)v.Nvt * v.Nx);
    const bool lo_t = e < 0.0;
    const double dth = fvm_band_row(lo_t ? v.vtL : v.vtR, v.ndt, v.Nvt, j, lo_t, X + (size_t)r * v.Nvt * v.Nx + x,
                                    (long long)v.Nx);
    const double adv = v.cos_t[j] * dr - dth / v.vr[r];
    const double col = G[(size_t)r * v.Nx + x] - v.loss[r] * z;
    return yx - c.dt * c.tau * (c.kappa * col + e * c.cA * adv);
}

// The collision inverse (I - c C)^-1 = D^-1 (x) I + (H (x) 1 w^T) at (r, j, x): T = H m, m the
// moments of B, (Nr, Nx)
FVM_HD double fvm_coll_apply_at(const FvmView& v, const double* dinv, const double* T, const double* B, int r, int j,
                                int x) {
    return dinv[r] * B[((size_t)r * v.Nvt + j) * v.Nx + x] + T[(size_t)r * v.Nx + x];
}

// ---------------------------------------------------------------------------------------
// Semi-Lagrangian advection (step_adv_vx_sl, bte_1d3v_solver.py:2244-2314): each value is the
// trilinear interpolant, on the grid padded by one layer in v_r and theta, at its departure
// point over one step; zero where the departure point leaves the padded grid.
// ---------------------------------------------------------------------------------------
struct FvmSl {
    int Nr, Nvt, Nx;
    const double* vr;     // Nr cell centres
    const double* vt;     // Nvt ordinates (pi ... 0)
    const double* cos_t;  // Nvt
    const double* vrp;    // Nr + 2: vmin, vr, vmax
    const double* vta;    // Nvt + 2: 0, vt reversed, pi (ascending)
    const double* x;      // Nx points, ascending
    double vmin;
    double cX;            // dt tau vth / L
    double cE;            // dt tau qe / (me vth)
};

// value of the padded grid at (a, b, x): a in [0, Nr + 1] along vrp, b in [0, Nvt + 1] along
// the reference's descending theta order (b = 0 is theta = pi); V (Nr, Nvt, Nx). The v_r = vmin
// layer and the theta = pi, 0 layers are linear extrapolations (:2286-2296); v_r = vmax is zero.
FVM_HD double fvm_sl_pad(const FvmSl& s, const double* V, int a, int b, int x) {
    const int Nr = s.Nr, Nvt = s.Nvt, Nx = s.Nx;
    if (a == Nr + 1) return 0.0;
    const double pi = 3.14159265358979323846;
    auto at = [&](int r, int j) { return V[((size_t)r * Nvt + j) * Nx + x]; };
    if (a >= 1) {
        const int r = a - 1;
        if (b >= 1 && b <= Nvt) return at(r, b - 1);
        if (b == 0) return at(r, 0) + (pi - s.vt[0]) * ((at(r, 1) - at(r, 0)) / (s.vt[1] - s.vt[0]));
        return at(r, Nvt - 1) - s.vt[Nvt - 1] * ((at(r, Nvt - 1) - at(r, Nvt - 2)) / (s.vt[Nvt - 1] - s.vt[Nvt - 2]));
    }
    const double cr = s.vr[0] - s.vmin, hr = s.vr[1] - s.vr[0];
    if (b >= 1 && b <= Nvt) return at(0, b - 1) - cr * ((at(1, b - 1) - at(0, b - 1)) / hr);
    if (b == 0)
        return at(0, 0) - cr * ((at(1, 0) - at(0, 0)) / hr) + (pi - s.vt[0]) * ((at(0, 1) - at(0, 0)) / (s.vt[1] - s.vt[0]));
    return at(0, Nvt - 1) - cr * ((at(1, Nvt - 1) - at(0, Nvt - 1)) / hr) -
           s.vt[Nvt - 1] * ((at(0, Nvt - 1) - at(0, Nvt - 2)) / (s.vt[Nvt - 1] - s.vt[Nvt - 2]));
}

// i in [0, n - 2] with g[i] < q <= g[i + 1] (i = 0 at q = g[0]) on an ascending grid of n points
FVM_HD int fvm_cell(const double* g, int n, double q) {
    int a = 0, b = n;
    while (a < b) {
        const int m = (a + b) >> 1;
        if (g[m] < q) a = m + 1;
        else b = m;
    }
    return a - 1 < 0 ? 0 : (a - 1 > n - 2 ? n - 2 : a - 1);
}

FVM_HD double fvm_sl_at(const FvmSl& s, const double* E, const double* V, int r, int j, int x) {
    const double vrc = s.vr[r] * s.cos_t[j];
    const double dE = s.cE * E[x];
    const double xa = s.x[x] - s.cX * vrc;
    const double va = sqrt(s.vr[r] * s.vr[r] + 2.0 * vrc * dE + dE * dE);
    // |cos| <= 1 up to rounding; held in [-1, 1] so that acos is defined
    const double ca = fmin(1.0, fmax(-1.0, (vrc + dE) / va));
    const double ta = acos(ca);
    const int nr = s.Nr + 2, nt = s.Nvt + 2;
    if (!(va >= s.vrp[0] && va <= s.vrp[nr - 1] && ta >= s.vta[0] && ta <= s.vta[nt - 1] && xa >= s.x[0] &&
          xa <= s.x[s.Nx - 1]))
        return 0.0;
    const int ir = fvm_cell(s.vrp, nr, va), it = fvm_cell(s.vta, nt, ta), ix = fvm_cell(s.x, s.Nx, xa);
    const double tr = (va - s.vrp[ir]) / (s.vrp[ir + 1] - s.vrp[ir]);
    const double tt = (ta - s.vta[it]) / (s.vta[it + 1] - s.vta[it]);
    const double tx = (xa - s.x[ix]) / (s.x[ix + 1] - s.x[ix]);
    double out = 0.0;
    for (int a = 0; a < 2; ++a) {
        const double wa = a ? tr : 1.0 - tr;
        for (int b = 0; b < 2; ++b) {
            const double wb = b ? tt : 1.0 - tt;
            const int bd = (nt - 1) - (it + b);   // ascending theta index -> the padded grid's order
            for (int c = 0; c < 2; ++c) {
                const double wc = c ? tx : 1.0 - tx;
                out += wa * wb * wc * fvm_sl_pad(s, V, ir + a, bd, ix + c);
            }
        }
    }
    return out;
}

// ---------------------------------------------------------------------------------------
// Restarted right-preconditioned GMRES(m) (the reference's utils.py:1172-1262 solves the same
// system): x0 = M^-1 b, classical Gram-Schmidt applied twice, Givens rotations, the residual
// recomputed at each restart. Ops supplies N, the vectors B (right-hand side), X (solution),
// R, W, Z, T (N each) and Kr (m + 1 vectors of N, contiguous), and
//   matvec(x, y), precond(x, y), dots(k, V, w, out_host[k]) (V: k vectors of N), sub_combo(k,
//   V, h_host, w) (w -= sum h_j V_j), combo(k, V, c_host, y) (y = sum c_j V_j), scale(a, x, y)
//   (y = a x, in place allowed), axpy(a, x, y), sub(a, b, c) (c = a - b);
// each returns 0 or an error code, which the solver returns at once.
// ---------------------------------------------------------------------------------------
struct FvmGmresInfo {
    int iterations;
    int converged;
    double rnorm, bnorm;
};

template <class Ops>
int fvm_gmres(Ops& op, int m, double rtol, double atol, int max_iter, FvmGmresInfo* info) {
    const size_t N = op.N;
    int rc;
    double bnorm = 0.0;
    if ((rc = op.dots(1, op.B, op.B, &bnorm))) return rc;
    bnorm = sqrt(bnorm);
    const double tol = std::max(atol, rtol * bnorm);
    if ((rc = op.precond(op.B, op.X))) return rc;
    int it = 0;
    double rnorm = 0.0;
    bool conv = false;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hh(m + 1), y(m);
    while (true) {
        if ((rc = op.matvec(op.X, op.W))) return rc;
        if ((rc = op.sub(op.B, op.W, op.R))) return rc;
        if ((rc = op.dots(1, op.R, op.R, &rnorm))) return rc;
        rnorm = sqrt(rnorm);
        if (rnorm <= tol) {
            conv = true;
            break;
        }
        if (it >= max_iter) break;
        if ((rc = op.scale(1.0 / rnorm, op.R, op.Kr))) return rc;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = rnorm;
        int k = 0;
        for (; k < m && it < max_iter; ++k, ++it) {
            double* vk = op.Kr + (size_t)k * N;
            double* vk1 = vk + N;
            if ((rc = op.precond(vk, op.Z))) return rc;
            if ((rc = op.matvec(op.Z, vk1))) return rc;
            for (int pass = 0; pass < 2; ++pass) {
                if ((rc = op.dots(k + 1, op.Kr, vk1, hh.data()))) return rc;
                if ((rc = op.sub_combo(k + 1, op.Kr, hh.data(), vk1))) return rc;
                for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = (pass == 0 ? 0.0 : H[(size_t)j * m + k]) + hh[j];
            }
            double nn = 0.0;
            if ((rc = op.dots(1, vk1, vk1, &nn))) return rc;
            nn = sqrt(nn);
            H[(size_t)(k + 1) * m + k] = nn;
            if (nn > 0.0 && (rc = op.scale(1.0 / nn, vk1, vk1))) return rc;
            for (int j = 0; j < k; ++j) {
                const double a = H[(size_t)j * m + k], b = H[(size_t)(j + 1) * m + k];
                H[(size_t)j * m + k] = cs[j] * a + sn[j] * b;
                H[(size_t)(j + 1) * m + k] = -sn[j] * a + cs[j] * b;
            }
            const double a = H[(size_t)k * m + k], b = H[(size_t)(k + 1) * m + k];
            const double rr = hypot(a, b);
            cs[k] = rr > 0.0 ? a / rr : 1.0;
            sn[k] = rr > 0.0 ? b / rr : 0.0;
            H[(size_t)k * m + k] = rr;
            H[(size_t)(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            if (fabs(g[k + 1]) <= tol || nn == 0.0) {
                ++k;
                ++it;
                break;
            }
        }
        for (int i = k - 1; i >= 0; --i) {
            double acc = g[i];
            for (int j = i + 1; j < k; ++j) acc -= H[(size_t)i * m + j] * y[j];
            y[i] = H[(size_t)i * m + i] != 0.0 ? acc / H[(size_t)i * m + i] : 0.0;
        }
        if ((rc = op.combo(k, op.Kr, y.data(), op.T))) return rc;
        if ((rc = op.precond(op.T, op.Z))) return rc;
        if ((rc = op.axpy(1.0, op.Z, op.X))) return rc;
    }
    info->iterations = it;
    info->converged = conv ? 1 : 0;
    info->rnorm = rnorm;
    info->bnorm = bnorm;
    return 0;
}

// Left-preconditioned restarted GMRES (the reference's gmres_pcl, utils.py:1266-1357): x0 = 0,
// the Krylov space of M^-1 A from M^-1 r0, and, as the reference does, the true residual
// ||b - A x|| of each iterate checked against max(atol, rtol ||b||) (one extra operator
// application per iteration). Same Ops as fvm_gmres.
template <class Ops>
int fvm_gmres_left(Ops& op, int m, double rtol, double atol, int max_iter, FvmGmresInfo* info) {
    const size_t N = op.N;
    int rc;
    double bnorm = 0.0;
    if ((rc = op.dots(1, op.B, op.B, &bnorm))) return rc;
    bnorm = sqrt(bnorm);
    const double tol = std::max(atol, rtol * bnorm);
    if ((rc = op.scale(0.0, op.B, op.X))) return rc;
    int it = 0;
    double rnorm = 0.0;
    bool conv = false;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hh(m + 1), y(m);
    auto solve_y = [&](int k) {
        for (int i = k - 1; i >= 0; --i) {
            double acc = g[i];
            for (int j = i + 1; j < k; ++j) acc -= H[(size_t)i * m + j] * y[j];
            y[i] = H[(size_t)i * m + i] != 0.0 ? acc / H[(size_t)i * m + i] : 0.0;
        }
    };
    while (true) {
        if ((rc = op.matvec(op.X, op.W))) return rc;
        if ((rc = op.sub(op.B, op.W, op.R))) return rc;
        if ((rc = op.dots(1, op.R, op.R, &rnorm))) return rc;
        rnorm = sqrt(rnorm);
        if (rnorm <= tol) {
            conv = true;
            break;
        }
        if (it >= max_iter) break;
        if ((rc = op.precond(op.R, op.Z))) return rc;
        double beta = 0.0;
        if ((rc = op.dots(1, op.Z, op.Z, &beta))) return rc;
        beta = sqrt(beta);
        if (!(beta > 0.0)) break;
        if ((rc = op.scale(1.0 / beta, op.Z, op.Kr))) return rc;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        bool done = false;
        for (; k < m && it < max_iter; ++k, ++it) {
            double* vk = op.Kr + (size_t)k * N;
            double* vk1 = vk + N;
            if ((rc = op.matvec(vk, op.W))) return rc;
            if ((rc = op.precond(op.W, vk1))) return rc;
            for (int pass = 0; pass < 2; ++pass) {
                if ((rc = op.dots(k + 1, op.Kr, vk1, hh.data()))) return rc;
                if ((rc = op.sub_combo(k + 1, op.Kr, hh.data(), vk1))) return rc;
                for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = (pass == 0 ? 0.0 : H[(size_t)j * m + k]) + hh[j];
            }
            double nn = 0.0;
            if ((rc = op.dots(1, vk1, vk1, &nn))) return rc;
            nn = sqrt(nn);
            H[(size_t)(k + 1) * m + k] = nn;
            if (nn > 0.0 && (rc = op.scale(1.0 / nn, vk1, vk1))) return rc;
            for (int j = 0; j < k; ++j) {
                const double a = H[(size_t)j * m + k], b = H[(size_t)(j + 1) * m + k];
                H[(size_t)j * m + k] = cs[j] * a + sn[j] * b;
                H[(size_t)(j + 1) * m + k] = -sn[j] * a + cs[j] * b;
            }
            const double a = H[(size_t)k * m + k], b = H[(size_t)(k + 1) * m + k];
            const double rr = hypot(a, b);
            cs[k] = rr > 0.0 ? a / rr : 1.0;
            sn[k] = rr > 0.0 ? b / rr : 0.0;
            H[(size_t)k * m + k] = rr;
            H[(size_t)(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            // the iterate x + V y and its true residual
            solve_y(k + 1);
            if ((rc = op.combo(k + 1, op.Kr, y.data(), op.T))) return rc;
            if ((rc = op.axpy(1.0, op.X, op.T))) return rc;
            if ((rc = op.matvec(op.T, op.W))) return rc;
            if ((rc = op.sub(op.B, op.W, op.R))) return rc;
            if ((rc = op.dots(1, op.R, op.R, &rnorm))) return rc;
            rnorm = sqrt(rnorm);
            if (rnorm <= tol || nn == 0.0) {
                ++k;
                ++it;
                done = rnorm <= tol;
                break;
            }
        }
        // restart from the last iterate
        if ((rc = op.scale(1.0, op.T, op.X))) return rc;
        if (done) {
            conv = true;
            break;
        }
    }
    info->iterations = it;
    info->converged = conv ? 1 : 0;
    info->rnorm = rnorm;
    info->bnorm = bnorm;
    return 0;
}
