// Galerkin assembly of the velocity-space operators on the device (FP64).
//
// Every kernel evaluates one operator entry (or one functional entry) per thread by
// summing over the Gauss points of the knot intervals where the integrand can be
// nonzero. The integrals are the reference's (file:line given per kernel); the
// reference loops over (p, k) pairs in Python processes, here each pair is a thread.
#include <vector>
#include <cmath>
#include <algorithm>
#include "bte_common.cuh"
#include "bte_grid.h"

static __device__ __host__ inline double c_gamma_d() { return sqrt(2.0 * (BTE_QE / BTE_ME)); }

// -------------------------------------------------------------------------------
// Quadrature tables: x, w and B-spline values / derivatives at every Gauss point of a
// per-interval rule (basis.py:414-429: x = 0.5 (b - a) gx + 0.5 (b + a), w = 0.5 (b - a) gw).
// -------------------------------------------------------------------------------
__global__ void k_quad_table(const double* __restrict__ t, int nsp, const int* __restrict__ iv_span,
                             const double* __restrict__ gx, const double* __restrict__ gw, int q, int npts,
                             double* x, double* w, int* span, double* B) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= npts) return;
    int iv = idx / q, g = idx % q;
    int j = iv_span[iv];
    double a = t[j], b = t[j + 1];
    double h = __dmul_rn(0.5, __dsub_rn(b, a));
    double xx = __dadd_rn(__dmul_rn(h, gx[g]), __dmul_rn(0.5, __dadd_rn(b, a)));
    x[idx] = xx;
    w[idx] = __dmul_rn(h, gw[g]);
    double d[3][4];
    int s = bspline_eval(t, nsp, xx, 2, d);
    span[idx] = s;
    for (int dd = 0; dd < 3; ++dd)
        for (int jj = 0; jj < 4; ++jj) B[(idx * 3 + dd) * 4 + jj] = d[dd][jj];
}

// value (derivative dd) of spline p at table point idx, 0 if p is not active there
__device__ inline double tabB(const double* B, const int* span, int idx, int p, int dd) {
    int j = p - (span[idx] - BTE_SP_ORDER);
    if (j < 0 || j > 3) return 0.0;
    return B[(idx * 3 + dd) * 4 + j];
}

// sigma of every process at the collision-rule points: eps = (x vth / c_gamma)^2
__global__ void k_sigma(const double* __restrict__ x, int npts, double vth, int nproc,
                        const int* __restrict__ off, const double* __restrict__ se,
                        const double* __restrict__ sv, double* sig) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    int pr = blockIdx.y;
    if (idx >= npts || pr >= nproc) return;
    double e = __ddiv_rn(__dmul_rn(x[idx], vth), c_gamma_d());
    e = __dmul_rn(e, e);
    int o = off[pr], m = off[pr + 1] - o;
    sig[pr * npts + idx] = interp_clamped(se + o, sv + o, m, e);
}

// Loop helper: points of rule (q points per interval) in knot spans [j0, j1].
#define FOR_SPAN_POINTS(iv_map, q, j0, j1, ...)                \
    for (int _j = (j0); _j <= (j1); ++_j) {                     \
        int _iv = iv_map[_j];                                   \
        if (_iv < 0) continue;                                  \
        for (int _g = 0; _g < (q); ++_g) {                      \
            int idx = _iv * (q) + _g;                           \
            __VA_ARGS__                                         \
        }                                                       \
    }

// Mass (spec_spherical.py:226-277) and CG advection radial blocks (:432-500), 10-point rule,
// banded storage [p][k - p + 3].
__global__ void k_mass_adv(int nsp, const int* __restrict__ iv_span, int q, const double* __restrict__ x,
                           const double* __restrict__ w, const int* __restrict__ span, const double* __restrict__ B,
                           double* Mr, double* mm1, double* mm2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int dk = blockIdx.y - BTE_BAND;
    if (p >= nsp) return;
    int k = p + dk;
    double s0 = 0, s1 = 0, s2 = 0;
    if (k >= 0 && k < nsp) {
        int j0 = max(p, k), j1 = min(p, k) + BTE_SP_ORDER;
        FOR_SPAN_POINTS(iv_span, q, j0, j1, {
            double xx = x[idx], ww = w[idx];
            double bp = tabB(B, span, idx, p, 0), bk = tabB(B, span, idx, k, 0), dbk = tabB(B, span, idx, k, 1);
            s0 += xx * xx * bp * bk * ww;
            s1 += xx * xx * bp * dbk * ww;
            s2 += xx * bp * bk * ww;
        })
    }
    Mr[p * BTE_NB + dk + BTE_BAND] = s0;
    mm1[p * BTE_NB + dk + BTE_BAND] = s1;
    mm2[p * BTE_NB + dk + BTE_BAND] = s2;
}

// Electron-heavy collision operator of one process, radial part
// (collision_operator_spherical.py:79-225):
//   q0[p][k] = sum_x w vth x^3 sigma phi_k(x) (split phi_p(v_post) - phi_p(x))   (l = 0)
//   q1[p][k] = -sum_x w vth x^3 sigma phi_k(x) phi_p(x)                          (l > 0)
// over the collision-rule points in supp(k), restricted to eps >= threshold for
// excitation / ionization. Accumulates into the species arrays.
__global__ void k_collision(int nsp, const double* __restrict__ t, const int* __restrict__ iv_span, int q,
                            const double* __restrict__ x, const double* __restrict__ w, const int* __restrict__ span,
                            const double* __restrict__ B, const double* __restrict__ sig, int gtype,
                            double threshold, double attach, double mByM, double vth,
                            double* q0, double* q1) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int p = blockIdx.y;
    if (k >= nsp) return;
    const double cg = c_gamma_d();
    double split = (gtype == BTE_PROC_IONIZATION) ? 2.0 : 1.0;
    double vscale = sqrt(1.0 - 2.0 * mByM);
    double a0 = 0.0, a1 = 0.0;
    bool band = abs(p - k) <= BTE_BAND;
    FOR_SPAN_POINTS(iv_span, q, k, k + BTE_SP_ORDER, {
        double xx = x[idx];
        double e = __ddiv_rn(__dmul_rn(xx, vth), cg);
        e = __dmul_rn(e, e);
        double vpost;
        bool keep = true;
        if (gtype == BTE_PROC_ELASTIC) {
            vpost = xx * vscale;
        } else if (gtype == BTE_PROC_ATTACHMENT) {
            vpost = cg * sqrt((1.0 / split) * (e + attach)) / vth;
        } else {
            keep = (e >= threshold);
            vpost = keep ? cg * sqrt((1.0 / split) * (e - threshold)) / vth : 0.0;
        }
        if (keep) {
            double base = w[idx] * vth * xx * xx * xx * sig[idx] * tabB(B, span, idx, k, 0);
            double pm = tabB(B, span, idx, p, 0);
            double pp = bspline_basis(t, nsp, p, vpost, 0);
            a0 += base * (split * pp - pm);
            if (band) a1 += -base * pm;
        }
    })
    q0[p * nsp + k] += a0;
    if (band) q1[p * BTE_NB + (k - p) + BTE_BAND] += a1;
}

// Gas-temperature operator, radial l = 0 block (collision_operator_spherical.py:443-498):
//   cgT[p][k] = -kappa sum_x w x^3 sigma_el phi_p'(x) phi_k'(x),  kappa = k_B (2 m/M) 0.5 / m_e / vth
__global__ void k_gas_temperature(int nsp, const int* __restrict__ iv_span, int q, const double* __restrict__ x,
                                  const double* __restrict__ w, const int* __restrict__ span,
                                  const double* __restrict__ B, const double* __restrict__ sig,
                                  double kappa, double* cgT) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int dk = blockIdx.y - BTE_BAND;
    if (p >= nsp) return;
    int k = p + dk;
    double s = 0.0;
    if (k >= 0 && k < nsp) {
        int j0 = max(p, k), j1 = min(p, k) + BTE_SP_ORDER;
        FOR_SPAN_POINTS(iv_span, q, j0, j1, {
            double xx = x[idx];
            s += w[idx] * (-kappa) * xx * xx * xx * sig[idx] * tabB(B, span, idx, p, 1) * tabB(B, span, idx, k, 1);
        })
    }
    cgT[p * BTE_NB + dk + BTE_BAND] += s;
}

// Radial functionals: sum over points of rule in supp(p) of w * x^e * f(x) * phi_p(x)
// mode 0: mass (utils.py:73-102)  1: temperature (:321-348)  2: mobility (:890-913)
// 3: diffusion (:915-944, 1/sigma_total)  4: rate of one process (:854-888)
__global__ void k_functional(int nsp, const int* __restrict__ iv_span, int q, const double* __restrict__ x,
                             const double* __restrict__ w, const int* __restrict__ span,
                             const double* __restrict__ B, int mode, const double* __restrict__ sig,
                             int nproc, int npts, double scale, double* out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nsp) return;
    double s = 0.0;
    FOR_SPAN_POINTS(iv_span, q, p, p + BTE_SP_ORDER, {
        double xx = x[idx];
        double bp = tabB(B, span, idx, p, 0);
        double v;
        if (mode == 0) v = xx * xx * bp;
        else if (mode == 1) v = xx * xx * xx * xx * bp;
        else if (mode == 2) v = xx * xx * xx * bp;
        else if (mode == 3) {
            double tot = 0.0;
            for (int pr = 0; pr < nproc; ++pr) tot += sig[pr * npts + idx];
            v = xx * xx * xx * bp / tot;
        } else v = xx * xx * xx * sig[idx] * bp;
        s += w[idx] * v;
    })
    out[p] = scale * s;
}

// Radial mass inverse by Cholesky, M^-1 = L^-T L^-1 (spec_spherical.py:299-336).
// One block; M is symmetric banded (|p - k| <= 3), L is dense lower in scratch.
__global__ void k_mass_inverse(int nsp, const double* __restrict__ Mr, double* L, double* Linv, double* Minv) {
    int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < nsp * nsp; i += nt) {
        int r = i / nsp, c = i % nsp;
        int d = c - r;
        L[i] = (d >= -BTE_BAND && d <= BTE_BAND) ? Mr[r * BTE_NB + d + BTE_BAND] : 0.0;
        Linv[i] = 0.0;
    }
    __syncthreads();
    // right-looking Cholesky on the lower triangle, column by column
    for (int j = 0; j < nsp; ++j) {
        __shared__ double djj;
        if (tid == 0) { djj = sqrt(L[j * nsp + j]); L[j * nsp + j] = djj; }
        __syncthreads();
        for (int i = j + 1 + tid; i < nsp; i += nt) L[i * nsp + j] /= djj;
        __syncthreads();
        for (int e = tid; e < (nsp - j - 1) * (nsp - j - 1); e += nt) {
            int r = j + 1 + e / (nsp - j - 1), c = j + 1 + e % (nsp - j - 1);
            if (c <= r) L[r * nsp + c] -= L[r * nsp + j] * L[c * nsp + j];
        }
        __syncthreads();
    }
    for (int i = tid; i < nsp * nsp; i += nt) {
        int r = i / nsp, c = i % nsp;
        if (c > r) L[i] = 0.0;
    }
    __syncthreads();
    // L^-1 column by column (forward substitution on unit vectors), one column per thread
    for (int c = tid; c < nsp; c += nt) {
        for (int r = c; r < nsp; ++r) {
            double s = (r == c) ? 1.0 : 0.0;
            for (int m = c; m < r; ++m) s -= L[r * nsp + m] * Linv[m * nsp + c];
            Linv[r * nsp + c] = s / L[r * nsp + r];
        }
    }
    __syncthreads();
    for (int i = tid; i < nsp * nsp; i += nt) {
        int r = i / nsp, c = i % nsp;
        double s = 0.0;
        for (int m = max(r, c); m < nsp; ++m) s += Linv[m * nsp + r] * Linv[m * nsp + c];
        Minv[i] = s;
    }
}

// Rosenbluth moment integrals (collision_operator_spherical.py:799-909):
//   mode 0 (P_m): int_{t_i}^{x_j} x^e B_i,  mode 1 (Q_m): int_{x_j}^{t_{i+4}} x^e B_i
// for the collision-rule points x_j inside supp(i) (local slot jj < 20) and, in slot 20,
// the integral over the whole support. Gauss rule gx/gw of the moment's order.
__global__ void k_moments(int nsp, const double* __restrict__ t, const int* __restrict__ iv_span, int q,
                          const double* __restrict__ x, int mode, int expo, const double* __restrict__ gx,
                          const double* __restrict__ gw, int ng, double* part, double* full) {
    int i = blockIdx.x;
    int jj = threadIdx.x;  // 0 .. 4q
    int nloc = 4 * q;
    if (i >= nsp || jj > nloc) return;
    double xb, xe;
    int slot = -1;
    if (jj == nloc) { xb = t[i]; xe = t[i + BTE_SP_ORDER + 1]; }
    else {
        int sj = i + jj / q, g = jj % q;
        int iv = iv_span[sj];
        if (iv < 0) { part[i * nloc + jj] = 0.0; return; }
        double xj = x[iv * q + g];
        slot = jj;
        if (mode == 0) { xb = t[i]; xe = xj; } else { xb = xj; xe = t[i + BTE_SP_ORDER + 1]; }
    }
    double acc = 0.0;
    for (int kn = i + 1; kn < i + BTE_SP_ORDER + 2; ++kn) {
        double a = fmax(xb, t[kn - 1]);
        double b = fmin(xe, t[kn]);
        if (b > a) {
            double s = 0.0;
            for (int g = 0; g < ng; ++g) {
                double qx = 0.5 * ((b - a) * gx[g] + (b + a));
                double qw = 0.5 * (b - a) * gw[g];
                double xp = (expo >= 0) ? pow(qx, (double)expo) : 1.0 / pow(qx, (double)(-expo));
                s += qw * xp * bspline_basis(t, nsp, i, qx, 0);
            }
            acc += s;
        }
    }
    if (slot >= 0) part[i * nloc + slot] = acc; else full[i] = acc;
}

struct MomentRef { const double* part; const double* full; };

// P or Q moment of spline k at collision-rule point (span sj, offset g)
__device__ inline double moment_at(const MomentRef& m, int mode, const double* t, int k, int sj, int g, int q, double xj) {
    int nloc = 4 * q;
    if (sj >= k && sj <= k + BTE_SP_ORDER) return m.part[k * nloc + (sj - k) * q + g];
    if (mode == 0) return (xj > t[k + BTE_SP_ORDER + 1]) ? m.full[k] : 0.0;
    return (xj < t[k]) ? m.full[k] : 0.0;
}

// hl / gl radial blocks for one l (collision_operator_spherical.py:911-969):
//   hl_l[p][k] = sum_j w_j x_j^2 B_p(x_j) m1_l(k, j),  gl_l likewise with m2_l.
__global__ void k_rosenbluth(int nsp, const double* __restrict__ t, const int* __restrict__ iv_span, int q,
                             const double* __restrict__ x, const double* __restrict__ w,
                             const int* __restrict__ span, const double* __restrict__ B, int l,
                             MomentRef Pl2, MomentRef Pl4, MomentRef Qlm1, MomentRef Qlm3,
                             double* hl, double* gl) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int p = blockIdx.y;
    if (k >= nsp) return;
    const double m_ab = 1.0;
    double ll = (double)l;
    double f1 = (ll - 0.5) / (ll + 1.5);
    double c1 = (2.0 / (2.0 * ll + 1.0)) * (1.0 + m_ab);
    double c2 = -(2.0 / (4.0 * ll * ll - 1.0));
    double sh = 0.0, sg = 0.0;
    for (int sj = p; sj <= p + BTE_SP_ORDER; ++sj) {
        int iv = iv_span[sj];
        if (iv < 0) continue;
        for (int g = 0; g < q; ++g) {
            int idx = iv * q + g;
            double xj = x[idx];
            double bp = tabB(B, span, idx, p, 0);
            double P2 = moment_at(Pl2, 0, t, k, sj, g, q, xj);
            double P4 = moment_at(Pl4, 0, t, k, sj, g, q, xj);
            double Q1 = moment_at(Qlm1, 1, t, k, sj, g, q, xj);
            double Q3 = moment_at(Qlm3, 1, t, k, sj, g, q, xj);
            double m1 = c1 * (P2 / pow(xj, ll + 1.0) + Q1 * pow(xj, ll));
            double m2 = c2 * ((P2 / pow(xj, ll - 1.0) - f1 * P4 / pow(xj, ll + 1.0))
                              + (Q3 * pow(xj, ll) - f1 * Q1 * pow(xj, ll + 2.0)));
            double wb = xj * xj * bp * w[idx];
            sh += wb * m1;
            sg += wb * m2;
        }
    }
    hl[p * nsp + k] = sh;
    gl[p * nsp + k] = sg;
}

// C = A B for small dense row-major nsp x nsp blocks (M^-1 times the raw hl / gl blocks)
__global__ void k_small_gemm(int nsp, const double* __restrict__ A, const double* __restrict__ Bm, double* C) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int r = blockIdx.y;
    if (c >= nsp) return;
    double s = 0.0;
    for (int m = 0; m < nsp; ++m) s += A[r * nsp + m] * Bm[m * nsp + c];
    C[r * nsp + c] = s;
}

// Coulomb radial integrals for (p, k = p + dk, r = p + dr) over the collision rule,
// combined with the angular tables into the trilinear coefficients
// (collision_operator_spherical.py:973-1120 with the weak forms of sym_cc.py:28-56):
//   CA[t] = 2 pi (R_a0 A1 + R_a1 A2)
//   CB[t] =   pi (R_b0 G0 + 2 R_b1 G1 + 2 R_b2 G0 + R_b3 G2 + R_b4 G3 + R_b5 G4)
__global__ void k_coulomb(int nsp, const int* __restrict__ iv_span, int q, const double* __restrict__ x,
                          const double* __restrict__ w, const int* __restrict__ span, const double* __restrict__ B,
                          int ntri, const double* __restrict__ angA, const double* __restrict__ angG,
                          double* CA, double* CB) {
    int p = blockIdx.x;
    int e = threadIdx.x;  // dk, dr pair
    if (p >= nsp || e >= BTE_NB * BTE_NB) return;
    int dk = e / BTE_NB - BTE_BAND, dr = e % BTE_NB - BTE_BAND;
    int k = p + dk, r = p + dr;
    double R[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (k >= 0 && k < nsp && r >= 0 && r < nsp && abs(k - r) <= BTE_BAND) {
        int j0 = max(p, max(k, r)), j1 = min(p, min(k, r)) + BTE_SP_ORDER;
        FOR_SPAN_POINTS(iv_span, q, j0, j1, {
            double xx = x[idx], iv = 1.0 / xx;
            double wk = w[idx] * tabB(B, span, idx, k, 0);
            double Bp = tabB(B, span, idx, p, 0), Dp = tabB(B, span, idx, p, 1), DDp = tabB(B, span, idx, p, 2);
            double Br = tabB(B, span, idx, r, 0), Dr = tabB(B, span, idx, r, 1), DDr = tabB(B, span, idx, r, 2);
            R[0] += wk * (xx * xx * Dp * Dr);
            R[1] += wk * (Bp * Br);
            R[2] += wk * (xx * xx * DDp * DDr);
            R[3] += wk * ((Dp - Bp * iv) * (Dr - Br * iv));
            R[4] += wk * (Dp * Dr);
            R[5] += wk * (Dp * Br * iv);
            R[6] += wk * (Bp * Dr * iv);
            R[7] += wk * (Bp * Br * iv * iv);
        })
    }
    for (int tt = 0; tt < ntri; ++tt) {
        const double* A = angA + 2 * tt;
        const double* G = angG + 5 * tt;
        double a = 2.0 * BTE_PI * (R[0] * A[0] + R[1] * A[1]);
        double b = BTE_PI * (R[2] * G[0] + 2.0 * R[3] * G[1] + 2.0 * R[4] * G[0] + R[5] * G[2] + R[6] * G[3] + R[7] * G[4]);
        size_t o = (((size_t)tt * nsp + p) * BTE_NB + (dk + BTE_BAND)) * BTE_NB + (dr + BTE_BAND);
        CA[o] = a;
        CB[o] = b;
    }
}

// Constraint and scaling vectors (bte_0d3v_batched.py:425-436, 636):
//   u = mass_op mw(0) vth^3, p = u / |u|, Mp = M p, W_s = u^T M^-1 C_s (l = 0 only).
__global__ void k_derived(int nsp, int nsh, int nspecies, double mw0, double vth, const double* __restrict__ mass,
                          const double* __restrict__ Mr, const double* __restrict__ Minv,
                          const double* __restrict__ q0, double* u, double* pv, double* Mp, double* W,
                          double* scratch) {
    __shared__ double red[32];
    int n = nsp * nsh, tid = threadIdx.x, nt = blockDim.x;
    double v3 = vth * vth * vth;
    double ss = 0.0;
    for (int a = tid; a < n; a += nt) {
        double ua = mass[a] * mw0 * v3;
        u[a] = ua;
        ss += ua * ua;
    }
    double nrm = sqrt(block_sum(ss, red));
    for (int a = tid; a < n; a += nt) pv[a] = u[a] / nrm;
    __syncthreads();
    for (int a = tid; a < n; a += nt) {
        int p = a / nsh, l = a % nsh;
        double s = 0.0;
        for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
            int k = p + dk;
            if (k >= 0 && k < nsp) s += Mr[p * BTE_NB + dk + BTE_BAND] * pv[k * nsh + l];
        }
        Mp[a] = s;
    }
    // scratch[p] = (M_r^-1 u_r)[p]
    for (int p = tid; p < nsp; p += nt) {
        double s = 0.0;
        for (int c = 0; c < nsp; ++c) s += Minv[p * nsp + c] * u[c * nsh];
        scratch[p] = s;
    }
    __syncthreads();
    for (int e = tid; e < nspecies * n; e += nt) {
        int sidx = e / n, a = e % n;
        int k = a / nsh, l = a % nsh;
        double s = 0.0;
        if (l == 0)
            for (int p = 0; p < nsp; ++p) s += scratch[p] * q0[((size_t)sidx * nsp + p) * nsp + k];
        W[e] = s;
    }
}

// merit vectors: invMd = 1 / diag(M), vD = D M p / |D M p|
__global__ void k_merit_vectors(int nsp, int nsh, const double* __restrict__ Mr, const double* __restrict__ Mp,
                                double* invMd, double* vD) {
    __shared__ double red[32];
    int n = nsp * nsh;
    double ss = 0.0;
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        double d = 1.0 / Mr[(a / nsh) * BTE_NB + BTE_BAND];
        invMd[a] = d;
        double v = Mp[a] * d;
        vD[a] = v;
        ss += v * v;
    }
    double nrm = sqrt(block_sum(ss, red));
    for (int a = threadIdx.x; a < n; a += blockDim.x) vD[a] /= nrm;
}

__global__ void k_to_float(const double* __restrict__ in, float* out, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

__global__ void k_absmax(const double* __restrict__ in, size_t n, double* out) {
    __shared__ double red[32];
    double m = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(in[i]));
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red[wid] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int i = 0; i < (int)((blockDim.x + 31) / 32); ++i) r = fmax(r, red[i]);
        *out = r;
    }
}

// -------------------------------------------------------------------------------
// host side
// -------------------------------------------------------------------------------
// Gauss-Legendre nodes/weights on [-1, 1], ascending (Newton iteration on the three-term
// recurrence of P_n from the Chebyshev-like initial guess; standard textbook method).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < (n + 1) / 2; ++i) {
        long double z = cosl(3.14159265358979323846264338327950288L * (i + 0.75L) / (n + 0.5L));
        long double pp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1.0L, p2 = 0.0L;
            for (int j = 1; j <= n; ++j) {
                long double p3 = p2;
                p2 = p1;
                p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0L);
            long double z1 = z;
            z = z1 - p1 / pp;
            if (fabsl(z - z1) < 1e-19L) break;
        }
        long double p1 = 1.0L, p2 = 0.0L;
        for (int j = 1; j <= n; ++j) {
            long double p3 = p2;
            p2 = p1;
            p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
        }
        pp = n * (z * p1 - p2) / (z * z - 1.0L);
        double wi = (double)(2.0L / ((1.0L - z * z) * pp * pp));
        x[i] = (double)(-z);
        x[n - 1 - i] = (double)z;
        w[i] = wi;
        w[n - 1 - i] = wi;
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

static int g_alloc(BteGrid* g, void** p, size_t bytes) {
    if (bytes == 0) bytes = 8;
    if (cudaMalloc(p, bytes) != cudaSuccess) return BTE_ERR_ALLOC;
    g->allocations.push_back(*p);
    cudaMemset(*p, 0, bytes);
    return BTE_OK;
}
#define GALLOC(ptr, count) do { if (g_alloc(g, (void**)&(ptr), sizeof(*(ptr)) * (size_t)(count))) return BTE_ERR_ALLOC; } while (0)
#define CK(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return BTE_ERR_CUDA; } while (0)

static int build_quad(BteGrid* g, BteQuad& Q, int q, cudaStream_t s) {
    std::vector<double> gx, gw;
    gauss_legendre(q, gx, gw);
    Q.q = q;
    Q.npts = g->nint * q;
    double *dgx, *dgw;
    GALLOC(dgx, q); GALLOC(dgw, q);
    GALLOC(Q.x, Q.npts); GALLOC(Q.w, Q.npts); GALLOC(Q.span, Q.npts); GALLOC(Q.B, (size_t)Q.npts * 12);
    std::vector<int> iv_span;
    for (int j = 0; j < (int)g->span_iv.size(); ++j) if (g->span_iv[j] >= 0) iv_span.push_back(j);
    int* d_iv_span;
    GALLOC(d_iv_span, iv_span.size());
    CK(cudaMemcpyAsync(d_iv_span, iv_span.data(), iv_span.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dgx, gx.data(), q * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dgw, gw.data(), q * sizeof(double), cudaMemcpyHostToDevice, s));
    k_quad_table<<<(Q.npts + 127) / 128, 128, 0, s>>>(g->d_t, g->nsp, d_iv_span, dgx, dgw, q, Q.npts, Q.x, Q.w, Q.span, Q.B);
    CK(cudaGetLastError());
    return BTE_OK;
}

static double sph_norm(int l) { return std::sqrt((2.0 * l + 1) / (4.0 * M_PI)); }

// Angular coefficients of the Coulomb weak forms (see k_coulomb): triples (q, l, s) with a
// nonzero coefficient, A = (A1, A2), G = (G0, G1, G2 - G5, G3 - G6, G4 + G7).
static void coulomb_angular(int lmax, std::vector<int>& tri, std::vector<double>& A, std::vector<double>& G) {
    int nq = 3 * lmax + 8;
    std::vector<double> mu, wq;
    gauss_legendre(nq, mu, wq);
    int L = lmax + 1;
    std::vector<double> Y(L * nq), dY(L * nq), Z(L * nq);
    for (int i = 0; i < nq; ++i) {
        double m = mu[i];
        double p0 = 1.0, p1 = m, d0 = 0.0, d1 = 1.0;
        for (int l = 0; l < L; ++l) {
            double P, D;
            if (l == 0) { P = 1.0; D = 0.0; }
            else if (l == 1) { P = m; D = 1.0; }
            else {
                P = ((2.0 * l - 1.0) * m * p1 - (l - 1.0) * p0) / l;
                D = l * p1 + m * d1;  // P_l' = l P_{l-1} + mu P_{l-1}'
                p0 = p1; p1 = P; d0 = d1; d1 = D;
            }
            Y[l * nq + i] = P * sph_norm(l);
            dY[l * nq + i] = D * sph_norm(l);
        }
        (void)d0;
        for (int l = 0; l < L; ++l) Z[l * nq + i] = m * dY[l * nq + i] - l * (l + 1.0) * Y[l * nq + i];
    }
    tri.clear(); A.clear(); G.clear();
    for (int q = 0; q < L; ++q)
        for (int l = 0; l < L; ++l)
            for (int s = 0; s < L; ++s) {
                double A1 = 0, A2 = 0, G2 = 0, G3 = 0, G4 = 0, G5 = 0, G6 = 0, G7 = 0;
                for (int i = 0; i < nq; ++i) {
                    double m = mu[i], yl = Y[l * nq + i] * wq[i], a = 1.0 - m * m;
                    double yq = Y[q * nq + i], ys = Y[s * nq + i], dq = dY[q * nq + i], ds = dY[s * nq + i];
                    double zq = Z[q * nq + i], zs = Z[s * nq + i];
                    A1 += yq * ys * yl; A2 += a * dq * ds * yl;
                    G2 += yq * zs * yl; G3 += zq * ys * yl; G4 += zq * zs * yl;
                    G5 += yq * m * ds * yl; G6 += m * dq * ys * yl; G7 += m * m * dq * ds * yl;
                }
                double v[5] = {A1, A2, G2 - G5, G3 - G6, G4 + G7};
                double mx = 0;
                for (double vi : v) mx = std::max(mx, std::fabs(vi));
                if (mx > 1e-13) {
                    tri.push_back(q); tri.push_back(l); tri.push_back(s);
                    A.push_back(A1); A.push_back(A2);
                    G.push_back(A1); G.push_back(A2); G.push_back(G2 - G5); G.push_back(G3 - G6); G.push_back(G4 + G7);
                }
            }
}

static int moment_order(int m, int mult) { return (((BTE_SP_ORDER + std::abs(m) + 1) / 2) + 1) * mult; }

int bte_assemble(BteGrid* g, cudaStream_t s) {
    const int nsp = g->nsp, nsh = g->nsh, n = g->n;
    // knots to device, span -> interval map
    GALLOC(g->d_t, g->knots.size());
    CK(cudaMemcpyAsync(g->d_t, g->knots.data(), g->knots.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    GALLOC(g->d_span_iv, g->span_iv.size());
    CK(cudaMemcpyAsync(g->d_span_iv, g->span_iv.data(), g->span_iv.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (build_quad(g, g->q5, g->spline_qpts, s)) return BTE_ERR_CUDA;
    if (build_quad(g, g->q10, 2 * (BTE_SP_ORDER + 2), s)) return BTE_ERR_CUDA;
    if (build_quad(g, g->q12, 2 * (BTE_SP_ORDER + 3), s)) return BTE_ERR_CUDA;

    // sigma at the collision rule
    GALLOC(g->d_sig5, (size_t)g->nproc * g->q5.npts);
    {
        dim3 gr((g->q5.npts + 127) / 128, g->nproc);
        k_sigma<<<gr, 128, 0, s>>>(g->q5.x, g->q5.npts, g->vth, g->nproc, g->d_sig_off, g->d_sig_e, g->d_sig_v, g->d_sig5);
        CK(cudaGetLastError());
    }
    // mass and advection
    GALLOC(g->d_Mr, nsp * BTE_NB); GALLOC(g->d_mm1, nsp * BTE_NB); GALLOC(g->d_mm2, nsp * BTE_NB);
    {
        dim3 gr((nsp + 63) / 64, BTE_NB);
        k_mass_adv<<<gr, 64, 0, s>>>(nsp, g->d_span_iv, g->q10.q, g->q10.x, g->q10.w, g->q10.span, g->q10.B, g->d_Mr, g->d_mm1, g->d_mm2);
        CK(cudaGetLastError());
    }
    // collisions
    GALLOC(g->d_q0, (size_t)g->nspecies * nsp * nsp);
    GALLOC(g->d_q1, (size_t)g->nspecies * nsp * BTE_NB);
    GALLOC(g->d_cgT, nsp * BTE_NB);
    for (int pr = 0; pr < g->nproc; ++pr) {
        int sp = g->proc_species[pr];
        dim3 gr((nsp + 63) / 64, nsp);
        k_collision<<<gr, 64, 0, s>>>(nsp, g->d_t, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span, g->q5.B,
                                      g->d_sig5 + (size_t)pr * g->q5.npts, g->proc_type[pr], g->proc_threshold[pr],
                                      g->proc_attach[pr], g->mByM, g->vth,
                                      g->d_q0 + (size_t)sp * nsp * nsp, g->d_q1 + (size_t)sp * nsp * BTE_NB);
        CK(cudaGetLastError());
        if (g->proc_type[pr] == BTE_PROC_ELASTIC) {
            double kappa = (BTE_KB * 1.0 * (2.0 * g->mByM) * 0.5 / BTE_ME) / g->vth;
            dim3 gr2((nsp + 63) / 64, BTE_NB);
            k_gas_temperature<<<gr2, 64, 0, s>>>(nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span, g->q5.B,
                                                 g->d_sig5 + (size_t)pr * g->q5.npts, kappa, g->d_cgT);
            CK(cudaGetLastError());
        }
    }
    // functionals
    GALLOC(g->d_mass, n); GALLOC(g->d_temp, n); GALLOC(g->d_mob, nsp); GALLOC(g->d_diff, nsp);
    GALLOC(g->d_rate, (size_t)g->nproc * nsp);
    {
        double* tmp;
        GALLOC(tmp, nsp);
        double sph_fac = sph_norm(0) * 4.0 * M_PI;
        const double cg = std::sqrt(2.0 * (BTE_QE / BTE_ME));
        const double K1EV = BTE_QE / BTE_KB;
        double v4 = std::pow(g->vth, 4);
        int nb = (nsp + 127) / 128;
        k_functional<<<nb, 128, 0, s>>>(nsp, g->d_span_iv, g->q10.q, g->q10.x, g->q10.w, g->q10.span, g->q10.B, 0, nullptr, 0, 0, sph_fac, tmp);
        CK(cudaMemcpy2DAsync(g->d_mass, nsh * sizeof(double), tmp, sizeof(double), sizeof(double), nsp, cudaMemcpyDeviceToDevice, s));
        double tscale = sph_fac * (0.5 * BTE_ME * (2.0 / 3.0 / BTE_KB) / K1EV);
        k_functional<<<nb, 128, 0, s>>>(nsp, g->d_span_iv, g->q12.q, g->q12.x, g->q12.w, g->q12.span, g->q12.B, 1, nullptr, 0, 0, tscale, tmp);
        CK(cudaMemcpy2DAsync(g->d_temp, nsh * sizeof(double), tmp, sizeof(double), sizeof(double), nsp, cudaMemcpyDeviceToDevice, s));
        k_functional<<<nb, 128, 0, s>>>(nsp, g->d_span_iv, g->q12.q, g->q12.x, g->q12.w, g->q12.span, g->q12.B, 2, nullptr, 0, 0, 2.0 * v4 / std::pow(cg, 4), g->d_mob);
        k_functional<<<nb, 128, 0, s>>>(nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span, g->q5.B, 3, g->d_sig5, g->nproc, g->q5.npts, 2.0 * v4 / std::pow(cg, 4), g->d_diff);
        for (int pr = 0; pr < g->nproc; ++pr)
            k_functional<<<nb, 128, 0, s>>>(nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span, g->q5.B, 4,
                                            g->d_sig5 + (size_t)pr * g->q5.npts, g->nproc, g->q5.npts, 2.0 * v4 / std::pow(cg, 3), g->d_rate + (size_t)pr * nsp);
        CK(cudaGetLastError());
    }
    // mass inverse
    GALLOC(g->d_Minv, (size_t)nsp * nsp);
    {
        double *L, *Li;
        GALLOC(L, (size_t)nsp * nsp); GALLOC(Li, (size_t)nsp * nsp);
        k_mass_inverse<<<1, 512, 0, s>>>(nsp, g->d_Mr, L, Li, g->d_Minv);
        CK(cudaGetLastError());
    }
    // advection angular coefficients (advection_operator_spherical_polys.py:12-16, m = 0)
    {
        std::vector<double> ac(nsh * 4, 0.0);
        for (int qq = 0; qq < nsh; ++qq) {
            if (qq + 1 <= g->lmax) {
                int l = qq + 1;
                ac[qq * 4 + 0] = (l) / (2.0 * l + 1.0) * sph_norm(l) / sph_norm(l - 1);
                ac[qq * 4 + 1] = (l) * (l + 1.0) / (2.0 * l + 1.0) * sph_norm(l) / sph_norm(l - 1);
            }
            if (qq - 1 >= 0) {
                int l = qq - 1;
                ac[qq * 4 + 2] = (l + 1.0) / (2.0 * l + 1.0) * sph_norm(l) / sph_norm(l + 1);
                ac[qq * 4 + 3] = -l * (l + 1.0) / (2.0 * l + 1.0) * sph_norm(l) / sph_norm(l + 1);
            }
        }
        GALLOC(g->d_adv_coef, nsh * 4);
        CK(cudaMemcpyAsync(g->d_adv_coef, ac.data(), ac.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    // constraint vectors
    GALLOC(g->d_u, n); GALLOC(g->d_p, n); GALLOC(g->d_Mp, n); GALLOC(g->d_W, (size_t)g->nspecies * n);
    {
        double* scratch;
        GALLOC(scratch, nsp);
        k_derived<<<1, 512, 0, s>>>(nsp, nsh, g->nspecies, g->mw0, g->vth, g->d_mass, g->d_Mr, g->d_Minv, g->d_q0,
                                    g->d_u, g->d_p, g->d_Mp, g->d_W, scratch);
        CK(cudaGetLastError());
        GALLOC(g->d_invMd, n); GALLOC(g->d_vD, n);
        k_merit_vectors<<<1, 512, 0, s>>>(nsp, nsh, g->d_Mr, g->d_Mp, g->d_invMd, g->d_vD);
        CK(cudaGetLastError());
    }
    // Coulomb operators
    if (g->ee) {
        coulomb_angular(g->lmax, g->tri, g->angA, g->angG);
        g->ntri = (int)g->tri.size() / 3;
        double *dA, *dG;
        GALLOC(dA, g->angA.size()); GALLOC(dG, g->angG.size()); GALLOC(g->d_tri, g->tri.size());
        CK(cudaMemcpyAsync(dA, g->angA.data(), g->angA.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dG, g->angG.data(), g->angG.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(g->d_tri, g->tri.data(), g->tri.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        size_t csz = (size_t)g->ntri * nsp * BTE_NB * BTE_NB;
        GALLOC(g->d_CA, csz); GALLOC(g->d_CB, csz);
        k_coulomb<<<nsp, 64, 0, s>>>(nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span, g->q5.B, g->ntri, dA, dG, g->d_CA, g->d_CB);
        CK(cudaGetLastError());

        // Rosenbluth moments: P_{l+2}, P_{l+4}, Q_{l-1}, Q_{l-3} for l = 0..lmax
        int q = g->q5.q, nloc = 4 * q;
        struct Mom { int mode, m; double* part; double* full; };
        std::vector<Mom> moms;
        auto get = [&](int mode, int m) -> Mom* {
            for (auto& mm : moms) if (mm.mode == mode && mm.m == m) return &mm;
            return nullptr;
        };
        for (int l = 0; l <= g->lmax; ++l) {
            int need[4][2] = {{0, l + 2}, {0, l + 4}, {1, l - 1}, {1, l - 3}};
            for (auto& nd : need) {
                if (get(nd[0], nd[1])) continue;
                Mom mm{nd[0], nd[1], nullptr, nullptr};
                GALLOC(mm.part, (size_t)nsp * nloc); GALLOC(mm.full, nsp);
                int ord = moment_order(nd[1], nd[0] == 0 ? 4 : 32);
                std::vector<double> gx, gw;
                gauss_legendre(ord, gx, gw);
                double *dgx, *dgw;
                GALLOC(dgx, ord); GALLOC(dgw, ord);
                CK(cudaMemcpyAsync(dgx, gx.data(), ord * sizeof(double), cudaMemcpyHostToDevice, s));
                CK(cudaMemcpyAsync(dgw, gw.data(), ord * sizeof(double), cudaMemcpyHostToDevice, s));
                int expo = (nd[0] == 0) ? nd[1] : -nd[1];
                k_moments<<<nsp, nloc + 1, 0, s>>>(nsp, g->d_t, g->d_span_iv, q, g->q5.x, nd[0], expo, dgx, dgw, ord, mm.part, mm.full);
                CK(cudaGetLastError());
                moms.push_back(mm);
            }
        }
        double *hraw, *graw;
        GALLOC(hraw, (size_t)nsp * nsp); GALLOC(graw, (size_t)nsp * nsp);
        GALLOC(g->d_HL, (size_t)nsh * nsp * nsp); GALLOC(g->d_GL, (size_t)nsh * nsp * nsp);
        for (int l = 0; l <= g->lmax; ++l) {
            Mom* a = get(0, l + 2); Mom* b = get(0, l + 4); Mom* c = get(1, l - 1); Mom* d = get(1, l - 3);
            dim3 gr((nsp + 63) / 64, nsp);
            k_rosenbluth<<<gr, 64, 0, s>>>(nsp, g->d_t, g->d_span_iv, q, g->q5.x, g->q5.w, g->q5.span, g->q5.B, l,
                                           MomentRef{a->part, a->full}, MomentRef{b->part, b->full},
                                           MomentRef{c->part, c->full}, MomentRef{d->part, d->full}, hraw, graw);
            k_small_gemm<<<gr, 64, 0, s>>>(nsp, g->d_Minv, hraw, g->d_HL + (size_t)l * nsp * nsp);
            k_small_gemm<<<gr, 64, 0, s>>>(nsp, g->d_Minv, graw, g->d_GL + (size_t)l * nsp * nsp);
            CK(cudaGetLastError());
        }
    }
    // FP32 copies for the mixed-precision Jacobian
    auto tof = [&](const double* src, float*& dst, size_t cnt) -> int {
        GALLOC(dst, cnt);
        if (cnt) k_to_float<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(src, dst, cnt);
        return cudaGetLastError() == cudaSuccess ? BTE_OK : BTE_ERR_CUDA;
    };
    if (tof(g->d_q0, g->f_q0, (size_t)g->nspecies * nsp * nsp)) return BTE_ERR_CUDA;
    if (tof(g->d_q1, g->f_q1, (size_t)g->nspecies * nsp * BTE_NB)) return BTE_ERR_CUDA;
    if (tof(g->d_cgT, g->f_cgT, (size_t)nsp * BTE_NB)) return BTE_ERR_CUDA;
    if (tof(g->d_mm1, g->f_mm1, (size_t)nsp * BTE_NB)) return BTE_ERR_CUDA;
    if (tof(g->d_mm2, g->f_mm2, (size_t)nsp * BTE_NB)) return BTE_ERR_CUDA;
    if (tof(g->d_Mr, g->f_Mr, (size_t)nsp * BTE_NB)) return BTE_ERR_CUDA;
    if (g->ee) {
        if (tof(g->d_HL, g->f_HL, (size_t)nsh * nsp * nsp)) return BTE_ERR_CUDA;
        if (tof(g->d_GL, g->f_GL, (size_t)nsh * nsp * nsp)) return BTE_ERR_CUDA;
        size_t csz = (size_t)g->ntri * nsp * BTE_NB * BTE_NB;
        if (tof(g->d_CA, g->f_CA, csz)) return BTE_ERR_CUDA;
        if (tof(g->d_CB, g->f_CB, csz)) return BTE_ERR_CUDA;
    }
    // magnitudes for scaling the bordered system
    {
        double* m;
        GALLOC(m, 4);
        k_absmax<<<1, 256, 0, s>>>(g->d_q0, (size_t)g->nspecies * nsp * nsp, m + 0);
        k_absmax<<<1, 256, 0, s>>>(g->d_mm1, (size_t)nsp * BTE_NB, m + 1);
        k_absmax<<<1, 256, 0, s>>>(g->d_u, (size_t)n, m + 2);
        k_absmax<<<1, 256, 0, s>>>(g->d_Mp, (size_t)n, m + 3);
        double hm[4];
        CK(cudaMemcpyAsync(hm, m, sizeof(hm), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        g->q0max = hm[0]; g->advmax = hm[1]; g->umax = hm[2]; g->Mpmax = hm[3];
    }
    CK(cudaStreamSynchronize(s));
    return BTE_OK;
}
