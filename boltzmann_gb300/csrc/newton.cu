// Batched steady-state Newton solve of the 0D3V Boltzmann equation on the device.
//
// The reference (bte_0d3v_batched.py:882-979) solves Q^T M^-1 F(h) = 0 for
// h = u/(u.u) + Q fb with M^-1-scaled dense operators, a Jacobian that drops the
// rank-1 growth term, an explicit batched inverse and a batch-global loop. This
// library solves the same equations (same fixed point) in the bordered form
//      F_raw(h) - lambda M p = 0,    u . h = 1,
// with the raw (un-scaled, banded) operators F_raw = M F, the exact Jacobian
// (including -(M h) w^T and the Coulomb-logarithm derivative), an LU of the
// (n+1) x (n+1) bordered matrix, per-point Armijo backtracking on the reference's
// merit (a lumped-mass scaling of the reference's 1/2 ||Q^T M^-1 F||^2, :939-952) and
// per-point convergence.
//
//   residual   FP64 always (one CTA per point)
//   Jacobian   FP64 (plain) or FP32 (mixed) straight into the factorization buffer
//   LU         FP64 or FP32, right-hand side appended as column n+1
#include <cstdio>
#include <mutex>
#include <deque>
#include <vector>
#include <algorithm>
#include <cmath>
#include "bte_common.cuh"
#include "bte_grid.h"
#include "dd_arith.h"

template <typename T>
cudaError_t bte_lu_factor_t(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s, int kernel);
template <typename T>
cudaError_t bte_lu_solve_t(int P, int N, const T* A, int ld, long long stride, const int32_t* piv, T* b, int mode,
                           cudaStream_t s, const int32_t* mats = nullptr);

// device view of a grid (passed by value to kernels)
struct GridView {
    int nsp, nsh, n, lmax, nspecies, ntri;
    int tqmax;  // largest number of e-e triples (q, l, s) sharing one q
    double vth, mw0, c_adv, gam_c, k1ev;
    const double *Mr, *Minv, *mm1, *mm2, *q0, *q1, *cgT, *adv_coef;
    const double *mass, *temp, *u, *p, *Mp, *W;
    const double *invMd, *vD;  // 1 / diag(M) and the unit vector D M p of the merit
    const double *HL, *GL, *CA, *CB;
    const int* tri;
    const float *fq0, *fq1, *fcgT, *fmm1, *fmm2, *fMr, *fHL, *fGL, *fCA, *fCB;
};

struct PointParams {
    const double *n0, *ne, *Tg, *E, *ns;  // ns: n_species x P (species-major)
    int P;
    const int8_t* eept;  // per-point e-e switch (a serving engine's warm-start phase); null: the launch's `ee`
};

// per-point scalar slots
enum { SC_GAMMA = 0, SC_MU, SC_T0, SC_M0, SC_NE, SC_COUNT = 8 };

// Double-double accumulation (the residual of a point at its FP64 rounding floor): an exact
// product (fma) and a compensated sum per term, rounded once at the end of a row (dd_arith.h).

// One row (mode q, spline p) of F_raw in double-double: the terms of k_residual's FP64 rows
// (electron-heavy collisions, gas temperature, advection, growth, e-e) with the Rosenbluth
// products shh/sgg given as hi + lo. Returns the row and its U and M h parts, rounded.
__device__ void residual_row_dd(const GridView& g, const PointParams& pp, int pt, int ee, int q, int p,
                                const double* sh, const double* shh, const double* shl, const double* sgg,
                                const double* sgl, double n0, double Tg, double cadv, double mu, double negam,
                                double& y, double& Uo, double& mho) {
    const int nsh = g.nsh, nsp = g.nsp;
    double yh = 0.0, yl = 0.0;
    for (int s = 0; s < g.nspecies; ++s) {
        const double ns = n0 * pp.ns[(size_t)s * pp.P + pt];
        double ah = 0.0, al = 0.0;
        if (q == 0) {
            const double* row = g.q0 + ((size_t)s * nsp + p) * nsp;
            for (int k = 0; k < nsp; ++k) dd_acc(ah, al, row[k], sh[k * nsh]);
        } else {
            const double* row = g.q1 + ((size_t)s * nsp + p) * BTE_NB;
            for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
                const int k = p + dk;
                if (k >= 0 && k < nsp) dd_acc(ah, al, row[dk + BTE_BAND], sh[k * nsh + q]);
            }
        }
        dd_acc2(yh, yl, ah, al, ns);
    }
    double gh = 0.0, gl = 0.0, vh = 0.0, vl = 0.0, mh = 0.0, ml = 0.0;
    for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
        const int k = p + dk;
        if (k < 0 || k >= nsp) continue;
        const int bi = p * BTE_NB + dk + BTE_BAND;
        if (q == 0) dd_acc(gh, gl, g.cgT[bi], sh[k * nsh]);
        if (q + 1 <= g.lmax) {
            const double a = g.mm1[bi] * g.adv_coef[q * 4 + 0] + g.adv_coef[q * 4 + 1] * g.mm2[bi];
            dd_acc(vh, vl, a, sh[k * nsh + q + 1]);
        }
        if (q >= 1) {
            const double a = g.mm1[bi] * g.adv_coef[q * 4 + 2] + g.adv_coef[q * 4 + 3] * g.mm2[bi];
            dd_acc(vh, vl, a, sh[k * nsh + q - 1]);
        }
        dd_acc(mh, ml, g.Mr[bi], sh[k * nsh + q]);
    }
    dd_acc2(yh, yl, gh, gl, n0 * Tg);
    dd_acc2(yh, yl, vh, vl, cadv);
    dd_acc2(yh, yl, mh, ml, -mu);
    double Uh = 0.0, Ul = 0.0;
    if (ee) {
        for (int t = 0; t < g.ntri; ++t) {
            if (g.tri[3 * t] != q) continue;
            const int l = g.tri[3 * t + 1], s = g.tri[3 * t + 2];
            const double* ca = g.CA + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
            const double* cb = g.CB + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
            for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
                const int k = p + dk;
                if (k < 0 || k >= nsp) continue;
                double ih = 0.0, il = 0.0;
                for (int dr = -BTE_BAND; dr <= BTE_BAND; ++dr) {
                    const int rr = p + dr;
                    if (rr < 0 || rr >= nsp) continue;
                    const int o = (dk + BTE_BAND) * BTE_NB + dr + BTE_BAND;
                    dd_acc2(ih, il, shh[rr * nsh + s], shl[rr * nsh + s], ca[o]);
                    dd_acc2(ih, il, sgg[rr * nsh + s], sgl[rr * nsh + s], cb[o]);
                }
                dd_acc2(Uh, Ul, ih, il, sh[k * nsh + l]);
            }
        }
        dd_acc2(yh, yl, Uh, Ul, negam);
    }
    y = yh + yl;
    Uo = Uh + Ul;
    mho = mh + ml;
}

// ---------------------------------------------------------------------------------
// Residual F_raw(h) for one point per CTA, plus ||(I - p p^T) M^-1 F_raw||.
// If dh != nullptr the CTA evaluates at h + alpha * dh and writes that state to hout.
// aux (if non-null) receives hh = HL h, gg = GL h, U = C_ee(h, h) raw, Mh = M h.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_residual(GridView g, PointParams pp, int ee, const int* __restrict__ act, int nact,
           const double* __restrict__ h, const double* __restrict__ dh, int ldd, const double* __restrict__ alpha,
           const int* __restrict__ need, double* hout, double* F, double* aux, double* scal, double* rnorm,
           double* srel, const int* __restrict__ ddm) {
    extern __shared__ double sm[];
    const int slot = blockIdx.x;
    if (slot >= nact) return;
    const int pt = act[slot];
    if (pp.eept) ee = pp.eept[pt];
    if (need && !need[pt]) return;
    // a point at its FP64 rounding floor is evaluated in double-double (smem 7 n instead of 5 n)
    const bool dd = ddm != nullptr && ddm[pt] != 0;
    const int n = g.n, nsh = g.nsh, nsp = g.nsp, tid = threadIdx.x, nt = blockDim.x;
    double* sh = sm;           // h
    double* shh = sm + n;      // HL h
    double* sgg = sm + 2 * n;  // GL h
    double* sF = sm + 3 * n;   // F_raw, later M^-1 F
    double* sR = sm + 4 * n;
    double* shl = sm + 5 * n;  // low parts of HL h and GL h (double-double points)
    double* sgl = sm + 6 * n;
    __shared__ double red[32];

    const double* hp = h + (size_t)pt * n;
    const double a = alpha ? alpha[pt] : 0.0;
    double sd = 0.0, shn = 0.0;
    for (int i = tid; i < n; i += nt) {
        double v = hp[i];
        if (dh) {
            double d = dh[(size_t)pt * ldd + i];
            sd += d * d;
            shn += v * v;
            v += a * d;
        }
        sh[i] = v;
        if (hout) hout[(size_t)pt * n + i] = v;
    }
    __syncthreads();
    if (srel) {
        sd = block_sum(sd, red);
        shn = block_sum(shn, red);
        if (tid == 0) srel[pt] = sqrt(sd / fmax(shn, 1e-300));
    }
    const double n0 = pp.n0[pt], Tg = pp.Tg[pt], E = pp.E[pt], ne = pp.ne[pt];
    double m0 = 0, t0 = 0, mu = 0;
    for (int i = tid; i < n; i += nt) {
        double v = sh[i];
        m0 += g.mass[i] * v;
        t0 += g.temp[i] * v;
        double ws = 0;
        for (int s = 0; s < g.nspecies; ++s) ws += n0 * pp.ns[(size_t)s * pp.P + pt] * g.W[(size_t)s * n + i];
        mu += ws * v;
    }
    m0 = block_sum(m0, red);
    t0 = block_sum(t0, red);
    mu = block_sum(mu, red);
    double gam = 0.0;
    if (ee) {
        for (int r = tid; r < n; r += nt) {
            int p = r / nsh, l = r % nsh;
            const double* HLr = g.HL + ((size_t)l * nsp + p) * nsp;
            const double* GLr = g.GL + ((size_t)l * nsp + p) * nsp;
            if (dd) {
                double h1 = 0, l1 = 0, h2 = 0, l2 = 0;
                for (int c = 0; c < nsp; ++c) {
                    const double hv = sh[c * nsh + l];
                    dd_acc(h1, l1, HLr[c], hv);
                    dd_acc(h2, l2, GLr[c], hv);
                }
                shh[r] = h1;
                shl[r] = l1;
                sgg[r] = h2;
                sgl[r] = l2;
                continue;
            }
            double s1 = 0, s2 = 0;
            for (int c = 0; c < nsp; ++c) {
                double hv = sh[c * nsh + l];
                s1 += HLr[c] * hv;
                s2 += GLr[c] * hv;
            }
            shh[r] = s1;
            sgg[r] = s2;
        }
        // Coulomb logarithm (bte_0d3v_batched.py:652-661)
        double mm0 = g.mw0 * m0 * g.vth * g.vth * g.vth;
        double kT = fabs(g.mw0 * ((t0 * g.k1ev) / mm0) * pow(g.vth, 5.0) * BTE_KB);
        double cl = (12.0 * BTE_PI * pow(BTE_EPS0 * kT, 1.5)) / (BTE_QE * BTE_QE * BTE_QE * sqrt(ne));
        gam = log(cl) * g.gam_c;
        __syncthreads();
    }
    const double cadv = E * g.c_adv;
    // rows mode-major: the lanes of a warp share the mode, so the dense l = 0 row and the
    // e-e triples of that mode run without divergence
    for (int rm = tid; rm < n; rm += nt) {
        const int q = rm / nsp, p = rm % nsp;
        const int r = p * nsh + q;
        if (dd) {
            double y, U, mh;
            residual_row_dd(g, pp, pt, ee, q, p, sh, shh, shl, sgg, sgl, n0, Tg, cadv, mu, ne * gam, y, U, mh);
            sF[r] = y;
            F[(size_t)pt * n + r] = y;
            if (aux) {
                double* ax = aux + (size_t)pt * 4 * n;
                ax[r] = shh[r] + shl[r];
                ax[n + r] = sgg[r] + sgl[r];
                ax[2 * n + r] = U;
                ax[3 * n + r] = mh;
            }
            continue;
        }
        double y = 0.0;
        // electron-heavy collisions
        for (int s = 0; s < g.nspecies; ++s) {
            double ns = n0 * pp.ns[(size_t)s * pp.P + pt];
            double acc = 0.0;
            if (q == 0) {
                const double* row = g.q0 + ((size_t)s * nsp + p) * nsp;
                for (int k = 0; k < nsp; ++k) acc += row[k] * sh[k * nsh];
            } else {
                const double* row = g.q1 + ((size_t)s * nsp + p) * BTE_NB;
                for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
                    int k = p + dk;
                    if (k >= 0 && k < nsp) acc += row[dk + BTE_BAND] * sh[k * nsh + q];
                }
            }
            y += ns * acc;
        }
        double gt = 0.0, adv = 0.0, mh = 0.0;
        for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
            int k = p + dk;
            if (k < 0 || k >= nsp) continue;
            int bi = p * BTE_NB + dk + BTE_BAND;
            if (q == 0) gt += g.cgT[bi] * sh[k * nsh];
            if (q + 1 <= g.lmax)
                adv += (g.mm1[bi] * g.adv_coef[q * 4 + 0] + g.adv_coef[q * 4 + 1] * g.mm2[bi]) * sh[k * nsh + q + 1];
            if (q >= 1)
                adv += (g.mm1[bi] * g.adv_coef[q * 4 + 2] + g.adv_coef[q * 4 + 3] * g.mm2[bi]) * sh[k * nsh + q - 1];
            mh += g.Mr[bi] * sh[k * nsh + q];
        }
        y += n0 * Tg * gt + cadv * adv - mu * mh;
        double U = 0.0;
        if (ee) {
            for (int t = 0; t < g.ntri; ++t) {
                if (g.tri[3 * t] != q) continue;
                const int l = g.tri[3 * t + 1], s = g.tri[3 * t + 2];
                const double* ca = g.CA + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
                const double* cb = g.CB + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
                for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
                    int k = p + dk;
                    if (k < 0 || k >= nsp) continue;
                    double inner = 0.0;
                    for (int dr = -BTE_BAND; dr <= BTE_BAND; ++dr) {
                        int rr = p + dr;
                        if (rr < 0 || rr >= nsp) continue;
                        int o = (dk + BTE_BAND) * BTE_NB + dr + BTE_BAND;
                        inner += ca[o] * shh[rr * nsh + s] + cb[o] * sgg[rr * nsh + s];
                    }
                    U += inner * sh[k * nsh + l];
                }
            }
            y += ne * gam * U;
        }
        sF[r] = y;
        F[(size_t)pt * n + r] = y;
        if (aux) {
            double* ax = aux + (size_t)pt * 4 * n;
            ax[r] = shh[r];
            ax[n + r] = sgg[r];
            ax[2 * n + r] = U;
            ax[3 * n + r] = mh;
        }
    }
    if (scal && tid == 0) {
        double* sc = scal + (size_t)pt * SC_COUNT;
        sc[SC_GAMMA] = gam; sc[SC_MU] = mu; sc[SC_T0] = t0; sc[SC_M0] = m0; sc[SC_NE] = ne;
    }
    __syncthreads();
    // merit ||P_v D F||, D = diag(M)^-1, v = D M p / |D M p|: zero exactly at the reference's
    // roots (Q^T M^-1 F = 0 <=> F || M p) without the round-off amplification of a dense M^-1
    double pr = 0.0;
    for (int r = tid; r < n; r += nt) {
        double d = sF[r] * g.invMd[r];
        sR[r] = d;
        pr += g.vD[r] * d;
    }
    pr = block_sum(pr, red);
    double nn = 0.0;
    for (int r = tid; r < n; r += nt) {
        double v = sR[r] - g.vD[r] * pr;
        nn += v * v;
    }
    nn = block_sum(nn, red);
    if (tid == 0) rnorm[pt] = sqrt(nn);
}

// The reference's merit ||(I - p p^T) M^-1 F|| = ||Q^T M^-1 F|| (bte_0d3v_batched.py:920-926)
// of stored raw residuals, for reporting (one CTA per point).
__global__ void __launch_bounds__(256)
k_ref_merit(GridView g, int P, const int* __restrict__ list, const double* __restrict__ F, double* out) {
    extern __shared__ double sm[];
    __shared__ double red[32];
    if ((int)blockIdx.x >= P) return;
    const int pt = list ? list[blockIdx.x] : (int)blockIdx.x;
    const int n = g.n, nsh = g.nsh, nsp = g.nsp, tid = threadIdx.x, nt = blockDim.x;
    double* sF = sm;
    double* sR = sm + n;
    for (int i = tid; i < n; i += nt) sF[i] = F[(size_t)pt * n + i];
    __syncthreads();
    double pr = 0.0;
    for (int r = tid; r < n; r += nt) {
        int p = r / nsh, l = r % nsh;
        const double* Mi = g.Minv + (size_t)p * nsp;
        double s = 0.0;
        for (int c = 0; c < nsp; ++c) s += Mi[c] * sF[c * nsh + l];
        sR[r] = s;
        pr += g.p[r] * s;
    }
    pr = block_sum(pr, red);
    double nn = 0.0;
    for (int r = tid; r < n; r += nt) {
        double v = sR[r] - g.p[r] * pr;
        nn += v * v;
    }
    nn = block_sum(nn, red);
    if (tid == 0) out[pt] = sqrt(nn);
}

// Per Jacobian row (p, q): K1 at the band columns (dk, s), e = (dk + 3) nsh + s, then
// K2a[s][dr] and K2b[s][dr] (the e-e bilinear form's two linearizations), in FP64.
__host__ __device__ inline int kc_row(int nsh) { return 3 * BTE_NB * nsh; }

// ---------------------------------------------------------------------------------
// FP64 iterative refinement of the mixed-precision Newton step: r = b - J x with the
// bordered Jacobian applied matrix-free in FP64 (the same terms k_jacobian writes):
//   (J x)[a] = static(x)[a] - mu (M x)[a] - (M h)[a] (w . x) + ne gamma [C(x; HL h, GL h)
//              + C(h; HL x, GL x)][a] + ne U[a] (dgamma . x) - beta Mp[a] x[n]
//   (J x)[n] = beta u . x,   b = (-F, beta (1 - u . h)).
// The residual is scaled by its max-norm sigma and stored in FP32 (slot-major) for the
// FP32 substitution; sigma[slot] is kept to undo the scaling.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_refine_residual(GridView g, PointParams pp, int ee, const int* __restrict__ act, int nact,
                  const double* __restrict__ h, const double* __restrict__ F, const double* __restrict__ aux,
                  const double* __restrict__ scal, const double* __restrict__ x, int ldd, double beta_scale,
                  const double* __restrict__ rowscale, float* __restrict__ rs, double* __restrict__ sigma,
                  const int* __restrict__ done, const double* __restrict__ kc, const int* __restrict__ slots,
                  int matvec, const double* __restrict__ xlist, int ldx, double* __restrict__ out64) {
    // slots (optional): CTA i works on slot slots[i]; xlist (optional): x of CTA i at
    // xlist + i * ldx instead of x[pt * ldd]; matvec: D (J x) instead of D (b - J x);
    // out64 (optional): the FP64 result of CTA i at out64 + i * (n + 1), and no FP32 output
    extern __shared__ double sm[];
    if ((int)blockIdx.x >= nact) return;
    const int slot = slots ? slots[blockIdx.x] : (int)blockIdx.x;
    const int pt = act[slot];
    if (pp.eept) ee = pp.eept[pt];
    const int n = g.n, nsh = g.nsh, nsp = g.nsp, N = n + 1, tid = threadIdx.x, nt = blockDim.x;
    if (done && done[pt]) {  // refinement finished for this point: a zero correction
        for (int i = tid; i < N; i += nt) rs[(size_t)slot * N + i] = 0.0f;
        if (tid == 0) sigma[slot] = 0.0;
        return;
    }
    double* sx = sm;            // x (n + 1)
    double* sh = sm + N;        // h
    double* sxh = sh + n;       // HL x
    double* sxg = sxh + n;      // GL x
    double* sr = sxg + n;       // r
    __shared__ double red[32];
    const double* hp = h + (size_t)pt * n;
    const double* ax = aux + (size_t)pt * 4 * n;
    const double* sc = scal + (size_t)pt * SC_COUNT;
    for (int i = tid; i < N; i += nt) sx[i] = xlist ? xlist[(size_t)blockIdx.x * ldx + i] : x[(size_t)pt * ldd + i];
    for (int i = tid; i < n; i += nt) sh[i] = hp[i];
    __syncthreads();
    const double n0 = pp.n0[pt], Tg = pp.Tg[pt], E = pp.E[pt], ne = sc[SC_NE];
    const double gam = sc[SC_GAMMA], mu = sc[SC_MU], t0 = sc[SC_T0], m0 = sc[SC_M0];
    const double beta = beta_scale * n0;
    double wx = 0, dgx = 0, ux = 0, uh = 0;
    for (int i = tid; i < n; i += nt) {
        double ws = 0;
        for (int s = 0; s < g.nspecies; ++s) ws += n0 * pp.ns[(size_t)s * pp.P + pt] * g.W[(size_t)s * n + i];
        wx += ws * sx[i];
        dgx += (g.temp[i] / t0 - g.mass[i] / m0) * sx[i];
        ux += g.u[i] * sx[i];
        uh += g.u[i] * sh[i];
    }
    wx = block_sum(wx, red);
    dgx = block_sum(dgx, red) * g.gam_c * 1.5;
    ux = block_sum(ux, red);
    uh = block_sum(uh, red);
    if (ee) {
        // HL x and GL x; rows taken mode-major so that a warp shares the mode
        for (int rm = tid; rm < n; rm += nt) {
            const int l = rm / nsp, p = rm % nsp;
            const double* HLr = g.HL + (size_t)rm * nsp;
            const double* GLr = g.GL + (size_t)rm * nsp;
            double s1 = 0, s2 = 0;
            for (int c = 0; c < nsp; ++c) {
                double v = sx[c * nsh + l];
                s1 += HLr[c] * v;
                s2 += GLr[c] * v;
            }
            sxh[p * nsh + l] = s1;
            sxg[p * nsh + l] = s2;
        }
        __syncthreads();
    }
    const double cadv = E * g.c_adv;
    const int kcn = kc_row(nsh);
    double amax = 0.0;
    // rows mode-major: the lanes of a warp take the same branch (dense l = 0 row or band)
    for (int rm = tid; rm < n; rm += nt) {
        const int q = rm / nsp, p = rm % nsp;
        const int r = p * nsh + q;
        double y = 0.0;
        for (int s = 0; s < g.nspecies; ++s) {
            double ns = n0 * pp.ns[(size_t)s * pp.P + pt];
            double acc = 0.0;
            if (q == 0) {
                const double* row = g.q0 + ((size_t)s * nsp + p) * nsp;
                for (int k = 0; k < nsp; ++k) acc += row[k] * sx[k * nsh];
            } else {
                const double* row = g.q1 + ((size_t)s * nsp + p) * BTE_NB;
                for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
                    int k = p + dk;
                    if (k >= 0 && k < nsp) acc += row[dk + BTE_BAND] * sx[k * nsh + q];
                }
            }
            y += ns * acc;
        }
        double gt = 0.0, adv = 0.0, mx = 0.0;
        for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
            int k = p + dk;
            if (k < 0 || k >= nsp) continue;
            int bi = p * BTE_NB + dk + BTE_BAND;
            if (q == 0) gt += g.cgT[bi] * sx[k * nsh];
            if (q + 1 <= g.lmax)
                adv += (g.mm1[bi] * g.adv_coef[q * 4 + 0] + g.adv_coef[q * 4 + 1] * g.mm2[bi]) * sx[k * nsh + q + 1];
            if (q >= 1)
                adv += (g.mm1[bi] * g.adv_coef[q * 4 + 2] + g.adv_coef[q * 4 + 3] * g.mm2[bi]) * sx[k * nsh + q - 1];
            mx += g.Mr[bi] * sx[k * nsh + q];
        }
        y += n0 * Tg * gt + cadv * adv - mu * mx - ax[3 * n + r] * wx;
        if (ee && kc) {
            // C(x; HL h, GL h) + C(h; HL x, GL x) through the row's coefficients, which the
            // Jacobian of this Newton step wrote: K1 . x over the band, K2a . (HL x) + K2b . (GL x)
            const double* kr = kc + ((size_t)slot * n + r) * kcn;
            double c1 = 0.0;
            for (int e = 0; e < BTE_NB * nsh; ++e) {
                const int k = p + e / nsh - BTE_BAND;
                if (k >= 0 && k < nsp) c1 += kr[e] * sx[k * nsh + e % nsh];
            }
            for (int e = 0; e < BTE_NB * nsh; ++e) {
                const int rr = p + e % BTE_NB - BTE_BAND;
                if (rr < 0 || rr >= nsp) continue;
                const int o = rr * nsh + e / BTE_NB;
                c1 += kr[BTE_NB * nsh + e] * sxh[o] + kr[2 * BTE_NB * nsh + e] * sxg[o];
            }
            y += ne * gam * c1 + ne * ax[2 * n + r] * dgx;
        }
        y += -beta * g.Mp[r] * sx[n];
        double rv = (matvec ? y : (-F[(size_t)pt * n + r] - y)) * rowscale[(size_t)slot * N + r];
        sr[r] = rv;
        amax = fmax(amax, fabs(rv));
    }
    if (tid == 0) {
        double rv = (matvec ? beta * ux : (beta * (1.0 - uh) - beta * ux)) * rowscale[(size_t)slot * N + n];
        sr[n] = rv;
        amax = fmax(amax, fabs(rv));
    }
    if (out64) {
        __syncthreads();
        for (int i = tid; i < N; i += nt) out64[(size_t)blockIdx.x * N + i] = sr[i];
        return;
    }
    // max-norm for the FP32 scaling
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = amax;
    __syncthreads();
    if (tid == 0) {
        double m = 0.0;
        for (int w = 0; w < (nt + 31) / 32; ++w) m = fmax(m, red[w]);
        red[0] = (m > 0.0) ? m : 1.0;
        sigma[slot] = red[0];
    }
    __syncthreads();
    const double inv = 1.0 / red[0];
    for (int i = tid; i < N; i += nt) rs[(size_t)slot * N + i] = (float)(sr[i] * inv);
}

// x[pt] += sigma * y[slot]; corr[pt] = ||sigma * y|| / ||x|| of this pass
__global__ void k_refine_update(int nact, const int* __restrict__ act, int N, const float* __restrict__ y,
                                const double* __restrict__ sigma, double* x, int ldd, double* corr,
                                const int* __restrict__ done) {
    __shared__ double red[32];
    int slot = blockIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (done[pt]) return;
    double sg = sigma[slot];
    double cc = 0.0, xx = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double d = sg * (double)y[(size_t)slot * N + i];
        double v = x[(size_t)pt * ldd + i] + d;
        x[(size_t)pt * ldd + i] = v;
        cc += d * d;
        xx += v * v;
    }
    cc = block_sum(cc, red);
    xx = block_sum(xx, red);
    if (threadIdx.x == 0) corr[pt] = sqrt(cc / fmax(xx, 1e-300));
}

// After refinement pass p >= 1 (0-based), per point: a correction at round-off or 4x
// smaller than the previous one ends the refinement; one that did not shrink (ratio
// above 0.9) means the FP32 factors cannot resolve this point's Jacobian: the point goes
// to the FP64 path. Otherwise keep refining (up to the pass limit).
__global__ void k_refine_check(int nact, const int* __restrict__ act, const double* __restrict__ c_prev,
                               const double* __restrict__ c_cur, int* status, int* done, int last) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (done[pt]) return;
    double a = c_prev[pt], b = c_cur[pt];
    if (b <= 1e-13 || b <= 0.25 * a) { done[pt] = 1; return; }
    if (!(b <= 0.9 * a)) {
        if (status[pt] < 0) status[pt] = BTE_ST_NEED_FP64;
        done[pt] = 1;
        return;
    }
    if (last) done[pt] = 1;
}

// After the first refinement pass: a correction below first_tol of the step means the FP32
// step was already accurate to ~first_tol (the corrected step to ~first_tol^2), so the
// refinement of this point ends; a point whose FP32 factors could not resolve its Jacobian
// shows a correction near 1, never this small.
__global__ void k_refine_first(int nact, const int* __restrict__ act, const double* __restrict__ c_cur, int* done,
                               double first_tol) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (!done[pt] && c_cur[pt] <= first_tol) done[pt] = 1;
}

// ---------------------------------------------------------------------------------
// GMRES refinement of the mixed-form Newton step for the points whose plain refinement
// stalled (the FP32 factors are then too inaccurate for a stationary iteration, but they
// still cluster the spectrum of the preconditioned operator): right-preconditioned
// GMRES(GM_M) on D J d = D b from d = 0, the preconditioner the FP32 LU substitution, the
// operator the matrix-free FP64 Jacobian (k_refine_residual in matvec mode), Arnoldi by
// classical Gram-Schmidt applied twice in FP64. The preconditioned vectors Z_k are kept, so
// the step is d = Z y (flexible form: the FP32 substitution need not be an exact linear
// map). A point whose residual falls below GM_TOL of ||D b|| ends; one above GM_ACCEPT of
// it after GM_M iterations is handed to the FP64 form. Lists: point i works on slot list[i].
// ---------------------------------------------------------------------------------
constexpr int GM_M = 20;
constexpr int GM_CAP = 512;  // points per GMRES batch
// GMRES refinement runs by default for bordered sizes above this. At c2's N = 385 it resolves
// all but 7 to 10 of the ~207 points per solve whose refinement stalls (9,350 to 9,590 against
// 9,150 solves/s with their FP64 factorizations), but it left 8 points 1e-7 to 8e-7 from
// plain FP64 (GM_TOL = 1e-8), where the FP64 hand-over keeps the mixed form's differences
// within FP64's own spread; a tighter GM_TOL (1e-12) helped at c2 but moved c5 points by up
// to 4e-2 (over-solving the flexible GMRES past its attainable accuracy).
constexpr int GM_MIN_N = 513;
// status of a point GMRES did not resolve, until all batches are done (k_gm_finalize makes it
// NEED_FP64); not negative, so the point is not running, and not NEED_FP64, so that a later
// batch does not collect it again
constexpr int GM_FAILED_MARK = 1000;
constexpr double GM_TOL = 1e-8;
constexpr double GM_ACCEPT = 1e-8;

// all: every running point as well (the diagnostic mode krylov = 2), first batch only
__global__ void k_gm_collect(int nact, const int* __restrict__ act, int* status, int* list, int* cnt, int cap,
                             bool all) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    const int pt = act[slot];
    if (status[pt] != BTE_ST_NEED_FP64 && !(all && status[pt] < 0)) return;
    const int i = atomicAdd(cnt, 1);
    if (i < cap) {
        list[i] = slot;
        status[pt] = -1;
    }
}

// v_0 = r_0 / ||r_0||, g = (||r_0||, 0, ...)
__global__ void k_gm_start(int ng, int N, const double* __restrict__ W, double* V, double* g, double* bn, int* on) {
    __shared__ double red[32];
    const int i = blockIdx.x;
    if (i >= ng) return;
    const double* w = W + (size_t)i * N;
    double ss = 0.0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) ss += w[j] * w[j];
    const double b = sqrt(block_sum(ss, red));
    const double inv = (b > 0.0) ? 1.0 / b : 0.0;
    double* v = V + (size_t)i * (GM_M + 1) * N;
    for (int j = threadIdx.x; j < N; j += blockDim.x) v[j] = w[j] * inv;
    if (threadIdx.x == 0) {
        bn[i] = b;
        g[(size_t)i * (GM_M + 1)] = b;
        on[i] = (b > 0.0) ? 1 : 0;
    }
}

// FP32 right-hand side of the substitution: v_k scaled by its max-norm
__global__ void k_gm_pre(int ng, int N, int k, const double* __restrict__ V, const int* __restrict__ on, float* xf,
                         double* sig) {
    __shared__ double red[32];
    const int i = blockIdx.x;
    if (i >= ng) return;
    const double* v = V + ((size_t)i * (GM_M + 1) + k) * N;
    float* x = xf + (size_t)i * N;
    if (!on[i]) {
        for (int j = threadIdx.x; j < N; j += blockDim.x) x[j] = 0.0f;
        return;
    }
    double m = 0.0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) m = fmax(m, fabs(v[j]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mm = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) mm = fmax(mm, red[w]);
        red[0] = (mm > 0.0) ? mm : 1.0;
        sig[i] = red[0];
    }
    __syncthreads();
    const double inv = 1.0 / red[0];
    for (int j = threadIdx.x; j < N; j += blockDim.x) x[j] = (float)(v[j] * inv);
}

// z_k = sigma * (FP32 substitution result), kept in FP64
__global__ void k_gm_post(int ng, int N, int k, const float* __restrict__ xf, const double* __restrict__ sig,
                          const int* __restrict__ on, double* Z) {
    const int i = blockIdx.x;
    if (i >= ng) return;
    double* z = Z + ((size_t)i * GM_M + k) * N;
    const double sg = on[i] ? sig[i] : 0.0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) z[j] = sg * (double)xf[(size_t)i * N + j];
}

__global__ void k_gm_finalize(int nact, const int* __restrict__ act, int* status) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    const int pt = act[slot];
    if (status[pt] == GM_FAILED_MARK) status[pt] = BTE_ST_NEED_FP64;
}

// One Arnoldi step on w = D J z_k, the Givens update of the least-squares problem, and for
// a point that ends, the step d = Z y written to dh (its status set when not accepted).
__global__ void __launch_bounds__(256)
k_gm_arnoldi(int ng, int N, int k, const double* __restrict__ W, double* V, double* H, double* cs, double* sn,
             double* g, const double* __restrict__ bn, int* on, const double* __restrict__ Z,
             const int* __restrict__ list, const int* __restrict__ act, double* dh, int ldd, int* status, int* active) {
    extern __shared__ double gw[];  // w (N)
    __shared__ double red[32];
    __shared__ double hc[GM_M + 2];
    __shared__ double yv[GM_M + 1];
    __shared__ int fin;
    const int i = blockIdx.x;
    if (i >= ng || !on[i]) return;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int j = tid; j < N; j += nt) gw[j] = W[(size_t)i * N + j];
    if (tid < GM_M + 2) hc[tid] = 0.0;
    __syncthreads();
    const double* Vi = V + (size_t)i * (GM_M + 1) * N;
    // classical Gram-Schmidt applied twice: all projections on the same w, then one update
    __shared__ double pc[GM_M + 1];
    for (int pass = 0; pass < 2; ++pass) {
        for (int j = 0; j <= k; ++j) {
            double d = 0.0;
            for (int t = tid; t < N; t += nt) d += Vi[(size_t)j * N + t] * gw[t];
            d = block_sum(d, red);
            if (tid == 0) pc[j] = d;
        }
        __syncthreads();
        for (int t = tid; t < N; t += nt) {
            double wt = gw[t];
            for (int j = 0; j <= k; ++j) wt -= pc[j] * Vi[(size_t)j * N + t];
            gw[t] = wt;
        }
        if (tid == 0)
            for (int j = 0; j <= k; ++j) hc[j] += pc[j];
        __syncthreads();
    }
    double ss = 0.0;
    for (int t = tid; t < N; t += nt) ss += gw[t] * gw[t];
    const double hk1 = sqrt(block_sum(ss, red));
    double* vk1 = V + ((size_t)i * (GM_M + 1) + k + 1) * N;
    const double inv = (hk1 > 0.0) ? 1.0 / hk1 : 0.0;
    for (int t = tid; t < N; t += nt) vk1[t] = gw[t] * inv;
    if (tid == 0) {
        double* csi = cs + (size_t)i * GM_M;
        double* sni = sn + (size_t)i * GM_M;
        double* gi = g + (size_t)i * (GM_M + 1);
        hc[k + 1] = hk1;
        for (int j = 0; j < k; ++j) {
            const double a = csi[j] * hc[j] + sni[j] * hc[j + 1];
            hc[j + 1] = -sni[j] * hc[j] + csi[j] * hc[j + 1];
            hc[j] = a;
        }
        const double den = hypot(hc[k], hc[k + 1]);
        const double c = (den > 0.0) ? hc[k] / den : 1.0, sv = (den > 0.0) ? hc[k + 1] / den : 0.0;
        csi[k] = c;
        sni[k] = sv;
        hc[k] = den;
        hc[k + 1] = 0.0;
        gi[k + 1] = -sv * gi[k];
        gi[k] = c * gi[k];
        double* Hi = H + ((size_t)i * GM_M + k) * (GM_M + 1);  // column k of R
        for (int j = 0; j <= k; ++j) Hi[j] = hc[j];
        const double res = fabs(gi[k + 1]);
        const bool ok = res <= GM_TOL * bn[i];
        fin = (ok || k == GM_M - 1 || !(hk1 > 0.0) || !isfinite(res)) ? 1 : 0;
        if (fin) {
            // back substitution R y = g over the k + 1 columns
            for (int j = k; j >= 0; --j) {
                double sacc = gi[j];
                for (int l = j + 1; l <= k; ++l) sacc -= H[((size_t)i * GM_M + l) * (GM_M + 1) + j] * yv[l];
                const double d = H[((size_t)i * GM_M + j) * (GM_M + 1) + j];
                yv[j] = (d != 0.0) ? sacc / d : 0.0;
            }
            const int pt = act[list[i]];
            if (!(res <= GM_ACCEPT * bn[i])) status[pt] = GM_FAILED_MARK;
            on[i] = 0;
        } else {
            atomicAdd(active, 1);
        }
    }
    __syncthreads();
    if (!fin) return;
    const int pt = act[list[i]];
    const double* Zi = Z + (size_t)i * GM_M * N;
    for (int t = tid; t < N; t += nt) {
        double x = 0.0;
        for (int j = 0; j <= k; ++j) x += yv[j] * Zi[(size_t)j * N + t];
        dh[(size_t)pt * ldd + t] = x;
    }
}

// ---------------------------------------------------------------------------------
// Bordered Jacobian, one warp per row, lanes along columns (row-major output), with the
// F_raw block scaled by jscale and jshift * M added (steady solve: 1, 0; transient backward
// Euler: -dt tau, 1):
//   J[a][j] = static(a, j) - mu M[a][j] - (M h)[a] w[j]
//             + ne gamma (K1[a][j] + (K2a HL)[a][j] + (K2b GL)[a][j]) + ne U[a] dgamma[j]
//   J[a][n] = -beta Mp[a] / Mpmax,   J[n][j] = beta u[j] / umax,   J[n][n] = 0
//   J[a][n+1] = -F[a],               J[n][n+1] = beta (1 - u.h) / umax
// ---------------------------------------------------------------------------------
template <typename T>
struct OpsT;
template <>
struct OpsT<double> {
    static __device__ const double* q0(const GridView& g) { return g.q0; }
    static __device__ const double* q1(const GridView& g) { return g.q1; }
    static __device__ const double* cgT(const GridView& g) { return g.cgT; }
    static __device__ const double* mm1(const GridView& g) { return g.mm1; }
    static __device__ const double* mm2(const GridView& g) { return g.mm2; }
    static __device__ const double* Mr(const GridView& g) { return g.Mr; }
    static __device__ const double* HL(const GridView& g) { return g.HL; }
    static __device__ const double* GL(const GridView& g) { return g.GL; }
    static __device__ const double* CA(const GridView& g) { return g.CA; }
    static __device__ const double* CB(const GridView& g) { return g.CB; }
};
template <>
struct OpsT<float> {
    static __device__ const float* q0(const GridView& g) { return g.fq0; }
    static __device__ const float* q1(const GridView& g) { return g.fq1; }
    static __device__ const float* cgT(const GridView& g) { return g.fcgT; }
    static __device__ const float* mm1(const GridView& g) { return g.fmm1; }
    static __device__ const float* mm2(const GridView& g) { return g.fmm2; }
    static __device__ const float* Mr(const GridView& g) { return g.fMr; }
    static __device__ const float* HL(const GridView& g) { return g.fHL; }
    static __device__ const float* GL(const GridView& g) { return g.fGL; }
    static __device__ const float* CA(const GridView& g) { return g.fCA; }
    static __device__ const float* CB(const GridView& g) { return g.fCB; }
};

constexpr int JAC_WARPS = 8;
constexpr int MIXED_HANDOVER_ITER = 30;  // mixed-form iterations before a running point moves to FP64

// Row equilibration of one bordered row (matrix part [0, N) and the RHS column N): the
// row is divided by its largest |entry| so that the factorization sees rows of unit
// size (the l = 0 energy-exchange rows are ~m/M smaller than the l >= 1 rows). The
// applied factor is returned for the FP64 refinement.
template <typename T>
__device__ inline void equilibrate_row(T* Jr, int N, int lane, double* scale_out) {
    T m = T(0);
    for (int j = lane; j < N; j += 32) m = fmax(m, fabs(Jr[j]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    const T sc = (m > T(0)) ? T(1) / m : T(1);
    for (int j = lane; j < N + 1; j += 32) Jr[j] *= sc;
    if (lane == 0 && scale_out) *scale_out = (double)sc;
}

// Byte offset of the staged HL / GL rows in k_jacobian's dynamic shared memory: before them
// sit the per-point column vectors of the l = 0 columns (FP64 W sums, their T copy, T copies
// of the temperature and mass rows) and the per-species scalars n0 * ns.
template <typename T>
__host__ __device__ inline size_t jac_col_bytes(int nsp, int nspecies) {
    return (((size_t)nsp + nspecies) * sizeof(double) + (size_t)3 * nsp * sizeof(T) + 15) & ~(size_t)15;
}
// then the per-warp partial sums of the e-e coefficients: tqmax triples x 7 offsets x
// (K2a, K2b, K1) in FP64
constexpr int JAC_TRI_MAX = 48;  // e-e triples of one mode (42 in all at l_max = 4)
__host__ __device__ inline size_t jac_part_bytes(int tqmax) {
    return (size_t)JAC_WARPS * tqmax * BTE_NB * 3 * sizeof(double);
}

// One bordered Jacobian row per warp. The row's entries fall in three groups, each
// handled by its own pass so that the lanes of a warp do the same work (an FP64
// instruction costs a full FP64-pipe slot however few lanes are active):
//   (1) l > 0 columns off the band: the dense Coulomb product only, T arithmetic;
//   (2) l = 0 columns off the band: rank-1 terms, plus the inelastic l = 0 block on
//       l = 0 rows, summed in FP64 there (they cancel nearly equal terms at low E/N);
//   (3) the band (p - 3 .. p + 3 splines x all modes): every term summed in FP64.
template <typename T>
__global__ void __launch_bounds__(JAC_WARPS * 32)
k_jacobian(GridView g, PointParams pp, int ee, const int* __restrict__ act, int nact, const double* __restrict__ h,
           const double* __restrict__ F, const double* __restrict__ aux, const double* __restrict__ scal,
           T* __restrict__ J, int ld, long long stride, double beta_scale, double* __restrict__ rowscale,
           int stage_hl, double jscale, double jshift, double* __restrict__ kc) {
    extern __shared__ __align__(16) unsigned char jsm[];
    const int slot = blockIdx.y;
    if (slot >= nact) return;
    const int pt = act[slot];
    if (pp.eept) ee = pp.eept[pt];
    const int n = g.n, nsh = g.nsh, nsp = g.nsp, N = n + 1, nspc = g.nspecies;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int a = blockIdx.x * JAC_WARPS + wid;  // row
    const double n0 = pp.n0[pt], Tg = pp.Tg[pt], E = pp.E[pt];
    // per-point column vectors of the l = 0 columns and the species scalars
    double* sWd = reinterpret_cast<double*>(jsm);
    double* sNs = sWd + nsp;
    T* sWt = reinterpret_cast<T*>(sNs + nspc);
    T* sTt = sWt + nsp;
    T* sMt = sTt + nsp;
    for (int sp = threadIdx.x; sp < nspc; sp += blockDim.x) sNs[sp] = n0 * pp.ns[(size_t)sp * pp.P + pt];
    for (int c = threadIdx.x; c < nsp; c += blockDim.x) {
        double w = 0.0;
        for (int sp = 0; sp < nspc; ++sp) w += n0 * pp.ns[(size_t)sp * pp.P + pt] * g.W[(size_t)sp * n + c * nsh];
        sWd[c] = w;
        sWt[c] = (T)w;
        sTt[c] = (T)g.temp[c * nsh];
        sMt[c] = (T)g.mass[c * nsh];
    }
    // rows of HL / GL this CTA's rows touch (p - 3 .. p + 3), staged in shared memory
    const int a0 = blockIdx.x * JAC_WARPS;
    const int prow0 = max(0, min(a0, n - 1) / nsh - BTE_BAND);
    const int prow1 = min(nsp - 1, min(a0 + JAC_WARPS - 1, n - 1) / nsh + BTE_BAND);
    const int nr = prow1 - prow0 + 1;
    double* part = reinterpret_cast<double*>(jsm + jac_col_bytes<T>(nsp, nspc)) + (size_t)wid * g.tqmax * BTE_NB * 3;
    T* sHL = reinterpret_cast<T*>(jsm + jac_col_bytes<T>(nsp, nspc) + jac_part_bytes(g.tqmax));
    T* sGL = sHL + (size_t)nr * nsh * nsp;
    if (stage_hl && ee) {
        const T* HLg = OpsT<T>::HL(g);
        const T* GLg = OpsT<T>::GL(g);
        for (int e = threadIdx.x; e < nr * nsh * nsp; e += blockDim.x) {
            const int sidx = e / (nr * nsp), rem = e % (nr * nsp);
            const size_t src = ((size_t)sidx * nsp + prow0 + rem / nsp) * nsp + rem % nsp;
            sHL[e] = HLg[src];
            sGL[e] = GLg[src];
        }
    }
    __syncthreads();
    if (a > n) return;
    T* Jr = J + (size_t)slot * stride + (size_t)a * ld;
    const double* hp = h + (size_t)pt * n;
    const double* ax = aux + (size_t)pt * 4 * n;
    const double* sc = scal + (size_t)pt * SC_COUNT;
    const bool be = (jshift != 0.0);
    // border scale: per unit n0 for the steady Jacobian (it matches the collision operator);
    // absolute for the backward-Euler matrix (it matches the mass matrix)
    const double beta = be ? beta_scale : beta_scale * n0;
    if (a == n) {  // constraint row
        double uh = 0.0;
        for (int j = lane; j < n; j += 32) {
            Jr[j] = (T)(beta * g.u[j]);
            uh += g.u[j] * hp[j];
        }
        uh = warp_sum(uh);
        if (lane == 0) {
            Jr[n] = T(0);
            Jr[n + 1] = (T)(beta * (1.0 - uh));
        }
        __syncwarp();
        equilibrate_row(Jr, N, lane, rowscale ? rowscale + (size_t)slot * N + a : nullptr);
        return;
    }
    const int p = a / nsh, q = a % nsh;
    const double ne = sc[SC_NE], gam = sc[SC_GAMMA], mu = sc[SC_MU], t0 = sc[SC_T0], m0 = sc[SC_M0];
    const double mh = ax[3 * n + a];
    const double Ua = ax[2 * n + a];
    const double negam = ee ? ne * gam : 0.0;
    // dgamma/dh = gam_c * 1.5 * (Top / (Top.h) - Mop / (Mop.h)), Top = temp * K_1eV
    const double dg_t = ee ? ne * Ua * g.gam_c * 1.5 / t0 : 0.0;
    const double dg_m = ee ? ne * Ua * g.gam_c * 1.5 / m0 : 0.0;
    // e-e coefficients of this row, in FP64 (the linearization of C(h; HL h, GL h)):
    //   K2a[s][dr] = sum_{t = (q, l, s)} sum_dk CA[t][p][dk][dr] h[(p + dk, l)]   (K2b: CB)
    //   K1[dk][s]  = sum_{t = (q, s, s')} sum_dr (CA[t][p][dk][dr] HLh[(p + dr, s')] + CB .. GLh)
    // One lane per (triple of mode q, offset) computes both partial sums, so that every lane
    // is busy; the partials are then summed over the triples in triple order. K2 is kept in
    // shared memory as T for the dense Coulomb product, K1 in FP64 for the band.
    __shared__ T k2s[JAC_WARPS][2][BTE_NB * 5];
    __shared__ double k1s[JAC_WARPS][BTE_NB * 5];
    __shared__ int tqs[JAC_WARPS][JAC_TRI_MAX];
    T* k2a = k2s[wid][0];
    T* k2b = k2s[wid][1];
    double* k1r = k1s[wid];
    int* tq = tqs[wid];
    double* kcr = (ee && kc) ? kc + ((size_t)slot * n + a) * kc_row(nsh) : nullptr;
    if (ee) {
        int ntq = 0;
        for (int t0 = 0; t0 < g.ntri; t0 += 32) {
            const int t = t0 + lane;
            const bool m = t < g.ntri && g.tri[3 * t] == q;
            const unsigned bal = __ballot_sync(0xffffffffu, m);
            const int at = ntq + __popc(bal & ((1u << lane) - 1u));
            if (m && at < JAC_TRI_MAX) tq[at] = t;
            ntq += __popc(bal);
        }
        ntq = min(ntq, g.tqmax);
        __syncwarp();
        for (int e = lane; e < ntq * BTE_NB; e += 32) {
            const int t = tq[e / BTE_NB], o = e % BTE_NB;
            const int l = g.tri[3 * t + 1], s2 = g.tri[3 * t + 2];
            const double* ca = g.CA + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
            const double* cb = g.CB + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
            double pa = 0.0, pb = 0.0, p1 = 0.0;
            for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {  // K2 partial, o = dr
                const int k = p + dk;
                if (k < 0 || k >= nsp) continue;
                const double hv = hp[k * nsh + l];
                pa += ca[(dk + BTE_BAND) * BTE_NB + o] * hv;
                pb += cb[(dk + BTE_BAND) * BTE_NB + o] * hv;
            }
            const int c = p + o - BTE_BAND;  // K1 partial, o = dk + 3
            if (c >= 0 && c < nsp) {
                for (int dr = -BTE_BAND; dr <= BTE_BAND; ++dr) {
                    const int rr = p + dr;
                    if (rr < 0 || rr >= nsp) continue;
                    p1 += ca[o * BTE_NB + dr + BTE_BAND] * ax[rr * nsh + s2] +
                          cb[o * BTE_NB + dr + BTE_BAND] * ax[n + rr * nsh + s2];
                }
            }
            part[3 * e + 0] = pa;
            part[3 * e + 1] = pb;
            part[3 * e + 2] = p1;
        }
        __syncwarp();
        for (int e = lane; e < nsh * BTE_NB; e += 32) {
            const int s = e / BTE_NB, dr = e % BTE_NB;     // K2[s][dr]
            const int dk3 = e / nsh, s1 = e % nsh;          // K1 at e = (dk + 3) nsh + s1
            double acc_a = 0.0, acc_b = 0.0, k1 = 0.0;
            for (int i = 0; i < ntq; ++i) {
                const int t = tq[i];
                if (g.tri[3 * t + 2] == s) {
                    acc_a += part[3 * (i * BTE_NB + dr) + 0];
                    acc_b += part[3 * (i * BTE_NB + dr) + 1];
                }
                if (g.tri[3 * t + 1] == s1) k1 += part[3 * (i * BTE_NB + dk3) + 2];
            }
            k2a[e] = (T)acc_a;
            k2b[e] = (T)acc_b;
            k1r[e] = k1;
            if (kcr) {
                kcr[e] = k1;
                kcr[BTE_NB * nsh + e] = acc_a;
                kcr[2 * BTE_NB * nsh + e] = acc_b;
            }
        }
        __syncwarp();
    }
    const T* HL = OpsT<T>::HL(g);
    const T* GL = OpsT<T>::GL(g);
    // dense Coulomb product of column (c, s) in T: sum_dr K2[s][dr] HL/GL[s][p + dr - 3][c]
    auto coulomb = [&](int c, int s) -> T {
        const T* hl = stage_hl ? sHL + ((ptrdiff_t)s * nr - prow0) * nsp + c : HL + (size_t)s * nsp * nsp + c;
        const T* gl = stage_hl ? sGL + ((ptrdiff_t)s * nr - prow0) * nsp + c : GL + (size_t)s * nsp * nsp + c;
        T acc = T(0);
#pragma unroll
        for (int dr = 0; dr < BTE_NB; ++dr) {
            int r = p + dr - BTE_BAND;
            if (r < 0 || r >= nsp) continue;
            acc += k2a[s * BTE_NB + dr] * hl[(size_t)r * nsp] + k2b[s * BTE_NB + dr] * gl[(size_t)r * nsp];
        }
        return acc;
    };
    const double cadv = E * g.c_adv;
    const T mh_t = (T)mh, negam_t = (T)negam, dgt_t = (T)dg_t, dgm_t = (T)dg_m, jscale_t = (T)jscale;
    if (lane == 0) {
        Jr[n] = (T)(-beta * g.Mp[a]);
        Jr[n + 1] = (T)(-F[(size_t)pt * n + a]);
    }
    // (1) l > 0 columns off the band
    const int nh = nsh - 1;
    for (int e = lane; e < nsp * nh; e += 32) {
        const int c = e / nh, s = 1 + e % nh;
        if (c >= p - BTE_BAND && c <= p + BTE_BAND) continue;
        T v = ee ? negam_t * coulomb(c, s) : T(0);
        Jr[c * nsh + s] = be ? v * jscale_t : v;
    }
    // (2) l = 0 columns off the band
    for (int c = lane; c < nsp; c += 32) {
        if (c >= p - BTE_BAND && c <= p + BTE_BAND) continue;
        const int j = c * nsh;
        const T acc = ee ? coulomb(c, 0) : T(0);
        if (q == 0) {
            double v = -mh * sWd[c];
            if (ee) {
                v += dg_t * g.temp[j] - dg_m * g.mass[j];
                v += negam * (double)acc;
            }
            const double* q0 = g.q0 + (size_t)p * nsp + c;
            for (int sp = 0; sp < nspc; ++sp) v += sNs[sp] * q0[(size_t)sp * nsp * nsp];
            if (be) v *= jscale;
            Jr[j] = (T)v;
        } else {
            T v = negam_t * acc;
            v += -mh_t * sWt[c];
            if (ee) v += dgt_t * sTt[c] - dgm_t * sMt[c];
            Jr[j] = be ? v * jscale_t : v;
        }
    }
    // (3) the band
    for (int e = lane; e < BTE_NB * nsh; e += 32) {
        const int dk = e / nsh - BTE_BAND, s = e % nsh;
        const int c = p + dk;
        if (c < 0 || c >= nsp) continue;
        const int j = c * nsh + s;
        const int bi = p * BTE_NB + dk + BTE_BAND;
        double v = 0.0;
        if (s == 0) {
            v = -mh * sWd[c];
            if (ee) v += dg_t * g.temp[j] - dg_m * g.mass[j];
        }
        if (ee) v += negam * (double)coulomb(c, s);
        if (s == q) {
            if (q == 0) {
                const double* q0 = g.q0 + (size_t)p * nsp + c;
                for (int sp = 0; sp < nspc; ++sp) v += sNs[sp] * q0[(size_t)sp * nsp * nsp];
                v += (n0 * Tg) * g.cgT[bi];
            } else {
                for (int sp = 0; sp < nspc; ++sp) v += sNs[sp] * g.q1[((size_t)sp * nsp + p) * BTE_NB + dk + BTE_BAND];
            }
            v -= mu * g.Mr[bi];
        }
        if (s == q + 1) v += cadv * (g.mm1[bi] * g.adv_coef[q * 4 + 0] + g.adv_coef[q * 4 + 1] * g.mm2[bi]);
        if (s == q - 1) v += cadv * (g.mm1[bi] * g.adv_coef[q * 4 + 2] + g.adv_coef[q * 4 + 3] * g.mm2[bi]);
        if (ee) v += negam * k1r[e];
        if (be) {  // backward-Euler form only: the steady kernel spends no FP64 op here
            v *= jscale;
            if (s == q) v += jshift * g.Mr[bi];
        }
        Jr[j] = (T)v;
    }
    __syncwarp();
    equilibrate_row(Jr, N, lane, rowscale ? rowscale + (size_t)slot * N + a : nullptr);
}

// h <- f / (u . f) (bte_0d3v_batched.py:903-911)
__global__ void k_mass_normalize(int n, const double* __restrict__ u, const double* __restrict__ f, double* h, int P) {
    __shared__ double red[32];
    int pt = blockIdx.x;
    if (pt >= P) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += u[i] * f[(size_t)pt * n + i];
    s = block_sum(s, red);
    for (int i = threadIdx.x; i < n; i += blockDim.x) h[(size_t)pt * n + i] = f[(size_t)pt * n + i] / s;
}

// ff / (mass / mm_fac . ff * 2 (vth / c_gamma)^3) (bte_0d3v_batched.py:1204-1217)
__global__ void k_normalized_distribution(int n, const double* __restrict__ mass, double mm_fac, double scale3,
                                          const double* __restrict__ h, double* f, int P) {
    __shared__ double red[32];
    int pt = blockIdx.x;
    if (pt >= P) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += (mass[i] / mm_fac) * h[(size_t)pt * n + i];
    s = block_sum(s, red) * scale3;
    for (int i = threadIdx.x; i < n; i += blockDim.x) f[(size_t)pt * n + i] = h[(size_t)pt * n + i] / s;
}

template <typename T>
__global__ void k_extract_step(int P_act, const int* __restrict__ act, const T* __restrict__ J, int ld,
                               long long stride, int N, double* dh, int ldd) {
    // the LU left x in column N (row-major, augmented): copy to a point-indexed FP64 buffer
    int slot = blockIdx.x;
    if (slot >= P_act) return;
    int pt = act[slot];
    for (int i = threadIdx.x; i < N; i += blockDim.x) dh[(size_t)pt * ldd + i] = (double)J[(size_t)slot * stride + (size_t)i * ld + N];
}

template <typename T>
__global__ void k_store_solution(int P_act, const T* __restrict__ xs, int N, const int* __restrict__ act, double* dh,
                                 int ldd) {
    int slot = blockIdx.x;
    if (slot >= P_act) return;
    int pt = act[slot];
    for (int i = threadIdx.x; i < N; i += blockDim.x) dh[(size_t)pt * ldd + i] = (double)xs[(size_t)slot * N + i];
}

// Armijo test (bte_0d3v_batched.py:942-952) for every point still searching. Round-off
// stop: a full Newton step smaller than step_rtol * ||h|| that does not decrease the merit
// (or a residual already below stagnate_rtol * ||r0|| that the full step cannot reduce)
// means the state is converged to the arithmetic's floor: for the worst-conditioned
// points of the batched workloads (cond ~ 5e10 after equilibration) the FP64 Newton steps
// at the floor are ~1e-9 of ||h||, so step_rtol = 1e-8 stops there. Where the floor's noise
// steps are larger than that, the search stalls instead: a merit already below
// STALL_RTOL * ||r0|| whose search has backtracked below STALL_ALPHA is at the floor (in the
// quadratic basin a Newton step is taken whole), and the point ends with stall_status
// (ROUNDOFF in FP64; the mixed form hands it to FP64) rather than halving on until a
// noise-level decrease passes the test at a vanishing step.
constexpr double STALL_ALPHA = 1.0 / 64.0;
constexpr double STALL_RTOL = 1e-6;
// A point whose merit stops resolving its steps at the FP64 rounding floor (the two ROUNDOFF
// exits below) while its Newton step is still above DD_STEP_RTOL of the state first switches
// its residual to double-double (ddm; ddpend asks the next Newton iteration to re-evaluate its
// state that way) and goes on; it ends at the double-double floor. A point whose step at the
// floor is already below DD_STEP_RTOL is resolved to FP64 precision in h and ends as before.
// Measured at c2 (4096 points): the largest mixed-vs-FP64 EDF difference fell from 9.6e-8 to
// 3.8e-9 (no point above 1e-8, 63 before) and FP64's own spread between two starting points
// from 9.3e-8 to 3.0e-8, for 18% of the mixed form's throughput (7,505 against 9,155 solves/s;
// switching every point at the floor cost 30%, a 1e-11 gate 23%).
constexpr double DD_STEP_RTOL = 1e-10;
__global__ void k_armijo(int nact, const int* __restrict__ act, int* searching, double* alpha,
                         const double* __restrict__ r, const double* __restrict__ rt, double c, double rho,
                         double amin, int* status, int* nsearch, int* accepted, const double* __restrict__ r0,
                         double stagnate_rtol, const double* __restrict__ srel, double step_rtol, int stall_status,
                         int* ddm, int* ddpend) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (!searching[pt]) return;
    if (status[pt] == BTE_ST_NEED_FP64) { searching[pt] = 0; accepted[pt] = 0; return; }
    double rr = r[pt], rn = rt[pt], al = alpha[pt];
    bool ok = (0.5 * rn * rn <= 0.5 * rr * rr - c * al * rr * rr);
    if (!isfinite(rn)) ok = false;
    const bool tiny = srel[pt] <= step_rtol;
    if (ok) {
        searching[pt] = 0;
        accepted[pt] = 1;
        // a step that barely contracts the merit at round-off level ends the solve after it is taken
        if (rn > 0.5 * rr && (rn <= stagnate_rtol * r0[pt] || srel[pt] <= 1e-2 * step_rtol)) {
            if (ddm && !ddm[pt] && srel[pt] > DD_STEP_RTOL) {
                ddm[pt] = 1;
                ddpend[pt] = 1;
            } else {
                status[pt] = BTE_ST_ROUNDOFF;
            }
        }
        return;
    }
    if (al == 1.0 && (rr <= stagnate_rtol * r0[pt] || tiny) && ddm && !ddm[pt] && srel[pt] > DD_STEP_RTOL) {
        searching[pt] = 0;
        accepted[pt] = 0;
        ddm[pt] = 1;
        ddpend[pt] = 1;
        return;
    }
    if (al == 1.0 && (rr <= stagnate_rtol * r0[pt] || tiny)) {
        // the merit no longer resolves the full step's effect: the solve ends without it.
        // (Taking a tiny last step anyway moved the Coulomb-dominated points of the c2-shape
        // fixture by their rounding floor, 1e-9, in either direction: no gain.)
        searching[pt] = 0;
        accepted[pt] = 0;
        status[pt] = BTE_ST_ROUNDOFF;
        return;
    }
    al *= rho;
    if (al < STALL_ALPHA && rr <= STALL_RTOL * r0[pt]) {
        searching[pt] = 0;
        accepted[pt] = 0;
        // a stalled search near the root may be the FP64 merit's noise: the point first goes
        // on with the double-double residual, as at the two ROUNDOFF exits
        if (ddm && !ddm[pt] && srel[pt] > DD_STEP_RTOL) {
            ddm[pt] = 1;
            ddpend[pt] = 1;
            return;
        }
        status[pt] = stall_status;
        return;
    }
    if (al < amin) {
        searching[pt] = 0;
        accepted[pt] = 0;
        status[pt] = BTE_ST_LINESEARCH;
        return;
    }
    alpha[pt] = al;
    atomicAdd(nsearch, 1);
}

__global__ void k_accept(int n, int nact, const int* __restrict__ act, const int* __restrict__ accepted,
                         double* h, const double* __restrict__ ht, double* F, const double* __restrict__ Ft,
                         double* aux, const double* __restrict__ auxt, double* scal, const double* __restrict__ scalt,
                         double* r, const double* __restrict__ rt, int* iters) {
    int slot = blockIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (!accepted[pt]) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        h[(size_t)pt * n + i] = ht[(size_t)pt * n + i];
        F[(size_t)pt * n + i] = Ft[(size_t)pt * n + i];
    }
    if (aux)
        for (int i = threadIdx.x; i < 4 * n; i += blockDim.x) aux[(size_t)pt * 4 * n + i] = auxt[(size_t)pt * 4 * n + i];
    if (threadIdx.x < SC_COUNT) scal[(size_t)pt * SC_COUNT + threadIdx.x] = scalt[(size_t)pt * SC_COUNT + threadIdx.x];
    if (threadIdx.x == 0) {
        r[pt] = rt[pt];
        iters[pt] += 1;
    }
}

// convergence test and compaction of the active list
// handover_iter > 0 (the mixed form): a point still running after that many iterations is
// handed to the FP64 form with the rest of its budget, so one slow point does not hold a
// whole batch in the mixed form until max_iter
__global__ void k_converge(int nact, const int* __restrict__ act, const double* __restrict__ r,
                           const double* __restrict__ r0, double atol, double rtol, int* nit, int max_iter,
                           int handover_iter, int* status, int* act_out, int* nout,
                           const int32_t* __restrict__ info, int check_info) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    int st = status[pt];
    const int it = ++nit[pt];  // Newton iterations of this point in its current solve
    if (st < 0) {
        if (!isfinite(r[pt])) st = BTE_ST_NONFINITE;
        else if (r[pt] <= atol + rtol * r0[pt]) st = BTE_ST_CONVERGED;
        else if (check_info && info[slot] != 0) st = BTE_ST_SINGULAR;
        else if (it >= max_iter) st = BTE_ST_MAXITER;
        else if (handover_iter > 0 && it >= handover_iter) st = BTE_ST_NEED_FP64;
        status[pt] = st;
    }
    if (st < 0) {
        int o = atomicAdd(nout, 1);
        act_out[o] = pt;
    }
}

__global__ void k_fill_int(int* p, int v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void k_set_list(int m, const int* __restrict__ list, int* a, int v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) a[list[i]] = v;
}
__global__ void k_iota(int* p, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}
__global__ void k_fill_dbl(double* p, double v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void k_set_active(int nact, const int* __restrict__ act, int* flag, double* alpha) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    flag[pt] = 1;
    alpha[pt] = 1.0;
}

// ---------------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------------
struct BteWork {
    int cap = 0, n = 0, prec = -1;
    size_t jbytes = 0;
    double *h = nullptr, *ht = nullptr, *F = nullptr, *Ft = nullptr, *aux = nullptr, *auxt = nullptr;
    double *scal = nullptr, *scalt = nullptr, *dh = nullptr, *r = nullptr, *rt = nullptr, *r0 = nullptr, *alpha = nullptr;
    double* xs = nullptr;  // LU solutions by slot, P x (n + 1)
    double* sigma = nullptr;  // refinement scaling by slot, P
    double* srel = nullptr;   // ||dh|| / ||h|| of the current Newton step, P
    double* rowscale = nullptr;  // row equilibration factors of the Jacobians, P x (n + 1)
    double* h0 = nullptr;     // initial state (restart of points that fall back to FP64), P x n
    double *ref_r = nullptr, *ref_r0 = nullptr;  // the reference's merit at the end / start, P
    double *corr0 = nullptr, *corr1 = nullptr;   // relative refinement corrections, first / last pass
    int32_t* reason = nullptr;                   // mixed-form status of each point before the FP64 pass
    int32_t *ddm = nullptr, *ddpend = nullptr;   // residual in double-double; its state to re-evaluate
    int32_t* refdone = nullptr;                  // refinement finished for the point in this Newton step
    int32_t* nit = nullptr;                      // Newton iterations of each point in its current solve
    void* J = nullptr;
    // e-e coefficients of the Jacobian rows in FP64 by slot (mixed form with e-e only):
    // P x n x kc_row(nsh), written by k_jacobian and applied by the refinement
    double* kc = nullptr;
    size_t kcbytes = 0;
    // GMRES refinement of stalled points (mixed form), gm_cap points at a time
    int gm_cap = 0;
    size_t gmbytes = 0;
    double *gm_V = nullptr, *gm_Z = nullptr, *gm_W = nullptr, *gm_H = nullptr, *gm_cs = nullptr, *gm_sn = nullptr;
    double *gm_g = nullptr, *gm_bn = nullptr, *gm_sig = nullptr;
    float* gm_xf = nullptr;
    int32_t *gm_list = nullptr, *gm_on = nullptr, *gm_cnt = nullptr;
    int32_t *piv = nullptr, *info = nullptr, *act = nullptr, *act2 = nullptr, *cnt = nullptr;
    int32_t *searching = nullptr, *accepted = nullptr;
};

static void free_work(BteWork* w) {
    void* ptrs[] = {w->nit, w->refdone, w->reason, w->ddm, w->ddpend, w->corr0, w->corr1, w->ref_r, w->ref_r0, w->rowscale, w->h0, w->srel, w->sigma, w->xs, w->h, w->ht, w->F, w->Ft, w->aux, w->auxt, w->scal, w->scalt, w->dh, w->r, w->rt, w->r0,
                    w->alpha, w->J, w->kc, w->gm_V, w->gm_Z, w->gm_W, w->gm_H, w->gm_cs, w->gm_sn, w->gm_g, w->gm_bn,
                    w->gm_sig, w->gm_xf, w->gm_list, w->gm_on, w->gm_cnt, w->piv, w->info, w->act, w->act2, w->cnt, w->searching, w->accepted};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    *w = BteWork();
}

static GridView view_of(const BteGrid* g) {
    GridView v;
    v.nsp = g->nsp; v.nsh = g->nsh; v.n = g->n; v.lmax = g->lmax; v.nspecies = g->nspecies; v.ntri = g->ntri;
    v.tqmax = 0;
    for (int q = 0; q < g->nsh; ++q) {
        int c = 0;
        for (int t = 0; t < g->ntri; ++t) c += (g->tri[3 * t] == q);
        v.tqmax = std::max(v.tqmax, c);
    }
    v.vth = g->vth; v.mw0 = g->mw0; v.c_adv = g->c_adv;
    v.gam_c = (BTE_QE * BTE_QE * BTE_QE * BTE_QE) / (4.0 * BTE_PI * (BTE_EPS0 * BTE_ME) * (BTE_EPS0 * BTE_ME)) / (g->vth * g->vth * g->vth);
    v.k1ev = BTE_QE / BTE_KB;
    v.Mr = g->d_Mr; v.Minv = g->d_Minv; v.mm1 = g->d_mm1; v.mm2 = g->d_mm2; v.q0 = g->d_q0; v.q1 = g->d_q1;
    v.cgT = g->d_cgT; v.adv_coef = g->d_adv_coef; v.mass = g->d_mass; v.temp = g->d_temp; v.u = g->d_u; v.p = g->d_p;
    v.Mp = g->d_Mp; v.W = g->d_W; v.invMd = g->d_invMd; v.vD = g->d_vD; v.HL = g->d_HL; v.GL = g->d_GL; v.CA = g->d_CA; v.CB = g->d_CB; v.tri = g->d_tri;
    v.fq0 = g->f_q0; v.fq1 = g->f_q1; v.fcgT = g->f_cgT; v.fmm1 = g->f_mm1; v.fmm2 = g->f_mm2; v.fMr = g->f_Mr;
    v.fHL = g->f_HL; v.fGL = g->f_GL; v.fCA = g->f_CA; v.fCB = g->f_CB;
    return v;
}

#define CKR(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { fprintf(stderr, "bte: %s at %s:%d\n", cudaGetErrorString(_e), __FILE__, __LINE__); return BTE_ERR_CUDA; } } while (0)

static int ensure_work(BteWork* w, const BteGrid* g, int P, int prec, int krylov = 0) {
    const int n = g->n, N = n + 1;
    const int ld = (N + 1 + 3) & ~3;  // row length of the augmented matrix, padded
    // the mixed form's FP64 pass reuses this buffer for FP64 matrices, half as many: it holds
    // at least two FP32 matrices so that one FP64 matrix fits whatever P is
    size_t jb = (prec == BTE_PREC_MIXED) ? (size_t)std::max(P, 2) * N * ld * sizeof(float)
                                         : (size_t)P * N * ld * sizeof(double);
    const size_t kb = (prec == BTE_PREC_MIXED && g->ee) ? (size_t)P * n * kc_row(g->nsh) * sizeof(double) : 0;
    const bool gm = prec == BTE_PREC_MIXED && (krylov > 0 || (krylov == 0 && N >= GM_MIN_N));
    const int gc = gm ? std::min(P, GM_CAP) : 0;
    const size_t gmb = (size_t)gc * (((size_t)(2 * GM_M + 2) * N + GM_M * (GM_M + 1) + 3 * GM_M + 4) * sizeof(double) +
                                     (size_t)N * sizeof(float) + 2 * sizeof(int32_t));
    if (w->cap >= P && w->n == n && w->jbytes >= jb && w->kcbytes >= kb && w->gm_cap >= gc) return BTE_OK;
    free_work(w);
    auto A = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, std::max<size_t>(bytes, 8)) == cudaSuccess; };
    size_t pn = (size_t)P * n * sizeof(double);
    bool ok = A((void**)&w->h, pn) && A((void**)&w->ht, pn) && A((void**)&w->F, pn) && A((void**)&w->Ft, pn) &&
              A((void**)&w->aux, 4 * pn) && A((void**)&w->auxt, 4 * pn) &&
              A((void**)&w->scal, (size_t)P * SC_COUNT * sizeof(double)) &&
              A((void**)&w->scalt, (size_t)P * SC_COUNT * sizeof(double)) &&
              A((void**)&w->dh, (size_t)P * (N + 1) * sizeof(double)) &&
              A((void**)&w->xs, (size_t)P * (N + 1) * sizeof(double)) &&
              A((void**)&w->sigma, (size_t)P * sizeof(double)) && A((void**)&w->srel, (size_t)P * sizeof(double)) &&
              A((void**)&w->rowscale, (size_t)P * (N + 1) * sizeof(double)) && A((void**)&w->h0, pn) &&
              A((void**)&w->ref_r, (size_t)P * sizeof(double)) && A((void**)&w->ref_r0, (size_t)P * sizeof(double)) &&
              A((void**)&w->corr0, (size_t)P * sizeof(double)) && A((void**)&w->corr1, (size_t)P * sizeof(double)) &&
              A((void**)&w->reason, (size_t)P * sizeof(int32_t)) && A((void**)&w->ddm, (size_t)P * sizeof(int32_t)) &&
              A((void**)&w->ddpend, (size_t)P * sizeof(int32_t)) && A((void**)&w->refdone, (size_t)P * sizeof(int32_t)) &&
              A((void**)&w->nit, (size_t)P * sizeof(int32_t)) && A((void**)&w->r, P * sizeof(double)) &&
              A((void**)&w->rt, P * sizeof(double)) && A((void**)&w->r0, P * sizeof(double)) &&
              A((void**)&w->alpha, P * sizeof(double)) && A(&w->J, jb) && (kb == 0 || A((void**)&w->kc, kb)) &&
              (gc == 0 || (A((void**)&w->gm_V, (size_t)gc * (GM_M + 1) * N * sizeof(double)) &&
                           A((void**)&w->gm_Z, (size_t)gc * GM_M * N * sizeof(double)) &&
                           A((void**)&w->gm_W, (size_t)gc * N * sizeof(double)) &&
                           A((void**)&w->gm_H, (size_t)gc * GM_M * (GM_M + 1) * sizeof(double)) &&
                           A((void**)&w->gm_cs, (size_t)gc * GM_M * sizeof(double)) &&
                           A((void**)&w->gm_sn, (size_t)gc * GM_M * sizeof(double)) &&
                           A((void**)&w->gm_g, (size_t)gc * (GM_M + 1) * sizeof(double)) &&
                           A((void**)&w->gm_bn, (size_t)gc * sizeof(double)) &&
                           A((void**)&w->gm_sig, (size_t)gc * sizeof(double)) &&
                           A((void**)&w->gm_xf, (size_t)gc * N * sizeof(float)) &&
                           A((void**)&w->gm_list, (size_t)gc * sizeof(int32_t)) &&
                           A((void**)&w->gm_on, (size_t)gc * sizeof(int32_t)) &&
                           A((void**)&w->gm_cnt, 4 * sizeof(int32_t)))) &&
              A((void**)&w->piv, (size_t)P * N * sizeof(int32_t)) && A((void**)&w->info, P * sizeof(int32_t)) &&
              A((void**)&w->act, P * sizeof(int32_t)) && A((void**)&w->act2, P * sizeof(int32_t)) &&
              A((void**)&w->cnt, 4 * sizeof(int32_t)) && A((void**)&w->searching, P * sizeof(int32_t)) &&
              A((void**)&w->accepted, P * sizeof(int32_t));
    if (!ok) { free_work(w); return BTE_ERR_ALLOC; }
    w->cap = P; w->n = n; w->jbytes = jb; w->kcbytes = kb; w->prec = prec;
    w->gm_cap = gc; w->gmbytes = gmb;
    return BTE_OK;
}

static inline unsigned nblk(int n, int b) { return (unsigned)((n + b - 1) / b); }

// Dynamic shared memory of k_jacobian: the per-point column vectors, and (with e-e on) the
// HL / GL rows of the CTA's splines when they fit in 96 KB (else they are read from HBM).
struct JacSmem {
    size_t bytes;
    int stage;
};
template <typename T>
static JacSmem jac_smem(const BteGrid* g, int ee) {
    int tqmax = 0;
    for (int q = 0; q < g->nsh; ++q) {
        int c = 0;
        for (int t = 0; t < g->ntri; ++t) c += (g->tri[3 * t] == q);
        tqmax = std::max(tqmax, c);
    }
    JacSmem r{jac_col_bytes<T>(g->nsp, g->nspecies) + jac_part_bytes(tqmax), 0};
    const int rows = (JAC_WARPS + g->nsh - 1) / g->nsh + 1 + 2 * BTE_BAND;
    const size_t hl = (size_t)2 * rows * g->nsh * g->nsp * sizeof(T);
    if (ee && r.bytes + hl <= 96 * 1024) {
        r.bytes += hl;
        r.stage = 1;
    }
    // above the default 48 KB the kernel's limit is raised (never lowered); a failure shows
    // at the launch
    bte_raise_smem_limit((const void*)k_jacobian<T>, r.bytes);
    return r;
}

BteWork* bte_work_get(BteGrid* g) {
    if (!g->work) g->work = new BteWork();
    return g->work;
}
void bte_work_release(BteWork* w) {
    if (w) { free_work(w); delete w; }
}

// ---------------------------------------------------------------------------------
// Library-wide launch counter and per-family CUDA-event timing (off unless enabled).
// ---------------------------------------------------------------------------------
enum { PF_RESIDUAL = 0, PF_JACOBIAN, PF_LU, PF_LUSOLVE, PF_REFINE, PF_OTHER, PF_LU64, PF_COUNT };
struct Profiler {
    // shared by every solve and serving engine of the process; engines driven from several
    // host threads record into it concurrently, so every member is guarded by `mu`
    std::mutex mu;
    bool on = false;
    long long launches = 0;
    long long fallback = 0;  // points of the mixed form re-solved in FP64
    long long fb_reason[8] = {0};  // ... by the status that sent them (2 max_iter .. 6 refinement)
    long long fam_launches[PF_COUNT] = {0};
    double fam_ms[PF_COUNT] = {0}, fam_flops[PF_COUNT] = {0}, fam_bytes[PF_COUNT] = {0};
    struct Rec { int fam; cudaStream_t s; cudaEvent_t a, b; double flops, bytes; };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t ev() {
        if (pool.empty()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            return e;
        }
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    // time one launch (or launch group) of family `fam` with algorithmic flops / bytes
    template <typename F>
    cudaError_t run(int fam, cudaStream_t s, double flops, double bytes, int nlaunch, F&& f) {
        std::lock_guard<std::mutex> lock(mu);
        launches += nlaunch;
        fam_launches[fam] += nlaunch;
        fam_flops[fam] += flops;
        fam_bytes[fam] += bytes;
        if (!on) { f(); return cudaGetLastError(); }
        Rec r{fam, s, ev(), ev(), flops, bytes};
        cudaEventRecord(r.a, s);
        f();
        cudaError_t e = cudaGetLastError();
        cudaEventRecord(r.b, s);
        pending.push_back(r);
        return e;
    }
    void count_fallback(long long n, const long long* reasons) {
        std::lock_guard<std::mutex> lock(mu);
        fallback += n;
        if (reasons)
            for (int i = 0; i < 8; ++i) fb_reason[i] += reasons[i];
    }
    void drain_locked(cudaStream_t s, bool all) {
        size_t keep = 0;
        for (size_t i = 0; i < pending.size(); ++i) {
            Rec& r = pending[i];
            if (!all && r.s != s) { pending[keep++] = r; continue; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, r.a, r.b);
            fam_ms[r.fam] += ms;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.resize(keep);
    }
    void drain(cudaStream_t s) {  // after stream `s` was synchronized: its records are complete
        std::lock_guard<std::mutex> lock(mu);
        drain_locked(s, false);
    }
    void reset(bool enable) {  // after a device synchronize
        std::lock_guard<std::mutex> lock(mu);
        drain_locked(nullptr, true);
        on = enable;
        launches = 0;
        fallback = 0;
        for (int i = 0; i < 8; ++i) fb_reason[i] = 0;
        for (int i = 0; i < PF_COUNT; ++i) { fam_launches[i] = 0; fam_ms[i] = 0; fam_flops[i] = 0; fam_bytes[i] = 0; }
    }
};
static Profiler g_prof;

extern "C" int bte_stats_reset(int enable_timing) {
    cudaDeviceSynchronize();
    g_prof.reset(enable_timing != 0);
    return BTE_OK;
}

// out[0] = kernel launches since the last reset; then for each family f in
// {residual, jacobian, lu_factor, lu_solve, refine, other, lu_factor_fp64}: launches, total
// ms (CUDA events, 0 when timing is off), algorithmic flops, algorithmic bytes; then the
// points of the mixed form re-solved in FP64 -> 2 + 4 * 7 doubles (+ 5 hand-over reasons).
extern "C" int bte_stats(double* out, int count) {
    if (!out || count < 2 + 4 * PF_COUNT) return BTE_ERR_ARG;
    cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lock(g_prof.mu);
    g_prof.drain_locked(nullptr, true);
    out[0] = (double)g_prof.launches;
    for (int f = 0; f < PF_COUNT; ++f) {
        out[1 + 4 * f] = (double)g_prof.fam_launches[f];
        out[2 + 4 * f] = g_prof.fam_ms[f];
        out[3 + 4 * f] = g_prof.fam_flops[f];
        out[4 + 4 * f] = g_prof.fam_bytes[f];
    }
    out[1 + 4 * PF_COUNT] = (double)g_prof.fallback;
    if (count >= 2 + 4 * PF_COUNT + 5)
        for (int i = 0; i < 5; ++i) out[2 + 4 * PF_COUNT + i] = (double)g_prof.fb_reason[2 + i];
    return BTE_OK;
}

// algorithmic work per point of each kernel family (flops; bytes moved to and from HBM)
static double res_flops_pt(const BteGrid* g, int ee) {
    double n = g->n, nsp = g->nsp, tri = g->ntri;
    double f = 2.0 * (nsp * nsp * g->nspecies + n * 7 * 4 + n * nsp);  // collisions, bands, M^-1 F
    if (ee) f += 2.0 * (2 * n * nsp) + 2.0 * 2.0 * nsp * tri * 49.0;   // potentials, trilinear form
    return f;
}
static double res_bytes_pt(const BteGrid* g, bool trial) {
    double n = g->n;
    return 8.0 * n * (1 + 1 + 4) + (trial ? 8.0 * (n + 1) + 8.0 * n : 0.0);  // h, F, aux (+ dh, h_trial)
}
static double jac_flops_pt(const BteGrid* g, int ee) {
    double n = g->n, N = n + 1;
    return ee ? 2.0 * (14.0 * n * n) + 4.0 * N * N : 4.0 * N * N;
}
static double lu_flops(int N) { return (2.0 / 3.0) * (double)N * N * N + (double)N * N; }

// points with status >= 2 (not converged) -> act list; their status reset to running
// A point's Newton budget (max_iter) covers both forms: a point that used it up in the
// mixed form ends with MAXITER; one whose line search, factorization or refinement failed
// (or whose residual became non-finite) continues in FP64 with the iterations it has left.
__global__ void k_collect_failed(int P, int* status, int* act_out, int* nout, int* reason) {
    int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= P) return;
    reason[pt] = status[pt];
    if (status[pt] >= BTE_ST_LINESEARCH) {
        status[pt] = -1;
        act_out[atomicAdd(nout, 1)] = pt;
    }
}

// A point handed to the FP64 form keeps its iteration count. It keeps its last accepted
// iterate when that iterate is already close to the root (merit below
// HANDOVER_KEEP_RTOL of the initial one): FP64 Newton finishes from there in a step or
// two. It restarts from h0 when its residual became non-finite, when its mixed-form
// trajectory went astray (its line search failed, or it was still running after
// MIXED_HANDOVER_ITER iterations; points converge in about 15), or when it is still far
// from the root. FP64 Newton was seen to stall for 90 iterations from a mixed iterate at 5%
// of the initial merit, while from h0 it converges in the iterations it always takes.
constexpr double HANDOVER_KEEP_RTOL = 1e-3;
__device__ inline bool handover_restarts(int reason, int nit, double r, double r0) {
    if (reason == BTE_ST_NONFINITE || reason == BTE_ST_LINESEARCH || nit >= MIXED_HANDOVER_ITER) return true;
    return !(r <= HANDOVER_KEEP_RTOL * r0);
}
__global__ void k_restore(int n, int nact, const int* __restrict__ act, const int* __restrict__ reason,
                          const double* __restrict__ h0, double* h, int* nit, const double* __restrict__ r,
                          const double* __restrict__ r0) {
    int slot = blockIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (!handover_restarts(reason[pt], nit[pt], r[pt], r0[pt])) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x) h[(size_t)pt * n + i] = h0[(size_t)pt * n + i];
}

struct SolveCtx {
    BteGrid* g;
    BteWork* w;
    GridView gv;
    PointParams pp;
    int P, n, N, ld, ldd, ee;
    long long jstride;
    double beta_scale;
    size_t res_smem, ref_smem;
    const bte_solve_opts* o;
    int32_t* status;
    int32_t* iters;
    cudaStream_t s;
};

// One active list of points and the buffers indexed by position in it (Jacobians, pivots,
// LU solutions, row scales, refinement scalings). A standalone solve runs one lane at a time;
// a serving engine keeps a mixed-precision lane and an FP64 lane.
struct Lane {
    int32_t *act, *act2;
    void* J;
    int32_t *piv, *info;
    double *xs, *rowscale, *sigma;
    double* kc;  // e-e row coefficients by slot (refined lanes), else null
};

// GMRES refinement (k_gm_*) of the points of lane L whose plain refinement stalled in this
// Newton iteration (status NEED_FP64 after the refinement passes), gm_cap points at a time.
// Each such point gets the step d = Z y from d = 0, or keeps NEED_FP64 when GMRES does not
// reach GM_ACCEPT. The Jacobian factors, row scales and e-e coefficients of the iteration
// are those the plain refinement used.
static cudaError_t gmres_refine(SolveCtx& c, Lane& L, int nact, bool all) {
    BteWork* w = c.w;
    const int N = c.N, ld = c.ld, ldd = c.ldd, ee = c.ee;
    cudaStream_t s = c.s;
    Profiler& pf = g_prof;
#define GMCK(x, what)                                                                            \
    do {                                                                                         \
        cudaError_t _e = (x);                                                                    \
        if (_e != cudaSuccess) {                                                                 \
            fprintf(stderr, "bte: GMRES refinement, %s: %s\n", what, cudaGetErrorString(_e));    \
            return _e;                                                                           \
        }                                                                                        \
    } while (0)
    for (int round = 0; round < 64; ++round) {
        GMCK(cudaMemsetAsync(w->gm_cnt, 0, 2 * sizeof(int32_t), s), "clear counters");
        k_gm_collect<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, c.status, w->gm_list, w->gm_cnt, w->gm_cap,
                                                     all && round == 0);
        GMCK(cudaGetLastError(), "collect");
        int hc[2] = {0, 0};
        GMCK(cudaMemcpyAsync(hc, w->gm_cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "read count");
        GMCK(cudaStreamSynchronize(s), "sync after collect");
        const int ng = std::min(hc[0], w->gm_cap);
        if (ng <= 0) break;
        const size_t zb = (size_t)ng * GM_M * N * sizeof(double);
        GMCK(pf.run(PF_REFINE, s, 0, 0, 2, [&] {
            // r0 = D b (d = 0): the first preconditioned vector is still zero
            cudaMemsetAsync(w->gm_Z, 0, zb, s);
            k_refine_residual<<<ng, 256, c.ref_smem, s>>>(c.gv, c.pp, ee, L.act, ng, w->h, w->F, w->aux, w->scal, w->dh,
                                                          ldd, c.beta_scale, L.rowscale, nullptr, nullptr, nullptr,
                                                          L.kc, w->gm_list, 0, w->gm_Z, GM_M * N, w->gm_W);
            k_gm_start<<<ng, 256, 0, s>>>(ng, N, w->gm_W, w->gm_V, w->gm_g, w->gm_bn, w->gm_on);
        }), "start");
        const size_t arn_smem = (size_t)N * sizeof(double);
        GMCK(bte_raise_smem_limit((const void*)k_gm_arnoldi, arn_smem), "shared memory limit");
        for (int k = 0; k < GM_M; ++k) {
            cudaError_t le = cudaSuccess;
            GMCK(pf.run(PF_REFINE, s, 0, 0, 5, [&] {
                k_gm_pre<<<ng, 256, 0, s>>>(ng, N, k, w->gm_V, w->gm_on, w->gm_xf, w->gm_sig);
                le = bte_lu_solve_t<float>(ng, N, (const float*)L.J, ld, c.jstride, L.piv, w->gm_xf, 0, s, w->gm_list);
                k_gm_post<<<ng, 256, 0, s>>>(ng, N, k, w->gm_xf, w->gm_sig, w->gm_on, w->gm_Z);
                k_refine_residual<<<ng, 256, c.ref_smem, s>>>(c.gv, c.pp, ee, L.act, ng, w->h, w->F, w->aux, w->scal,
                                                              w->dh, ldd, c.beta_scale, L.rowscale, nullptr, nullptr,
                                                              nullptr, L.kc, w->gm_list, 1, w->gm_Z + (size_t)k * N,
                                                              GM_M * N, w->gm_W);
                cudaMemsetAsync(w->gm_cnt + 1, 0, sizeof(int32_t), s);
                k_gm_arnoldi<<<ng, 256, arn_smem, s>>>(ng, N, k, w->gm_W, w->gm_V, w->gm_H, w->gm_cs, w->gm_sn, w->gm_g,
                                                       w->gm_bn, w->gm_on, w->gm_Z, w->gm_list, L.act, w->dh, ldd,
                                                       c.status, w->gm_cnt + 1);
            }), "iteration");
            GMCK(le, "substitution");
            int left = 0;
            GMCK(cudaMemcpyAsync(&left, w->gm_cnt + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "read active");
            GMCK(cudaStreamSynchronize(s), "sync after iteration");
            if (left == 0) break;
        }
        if (hc[0] <= w->gm_cap) break;  // every stalled point had a place in this batch
    }
#undef GMCK
    k_gm_finalize<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, c.status);
    return cudaGetLastError();
}

// FP32 factorization kernel for a Newton system of size N (bte_solve_opts.lu_kernel): a
// kernel that does not take N falls back to the library's choice
static int lu_kernel_for(int requested, int N) {
    if ((requested == 2 || requested == 3 || requested == 4 || requested == 5) && N > 512) return 0;
    return (requested >= 0 && requested <= 5) ? requested : 0;
}

// FP64 factorization kernel (bte_solve_opts.lu64_kernel): the split kernel unless the one-CTA
// kernel is asked for. A point's arithmetic does not depend on how many points share a launch
// with either kernel.
static int lu64_kernel_for(int requested) { return requested == 1 ? 1 : 6; }

// One Newton iteration (Jacobian, factorization, step, refinement, line search, acceptance,
// convergence test) for the `nact` points of lane L whose F, aux, scal and r are current;
// returns the points still running, whose list is then L.act (the list before the
// iteration is left in L.act2), or a negative code.
static int newton_iteration(SolveCtx& c, Lane& L, int nact, int prec) {
    BteGrid* g = c.g;
    BteWork* w = c.w;
    const int n = c.n, N = c.N, ld = c.ld, ldd = c.ldd, ee = c.ee, P = c.P;
    const long long jstride = c.jstride;
    const double beta_scale = c.beta_scale;
    const size_t res_smem = c.res_smem, ref_smem = c.ref_smem;
    const bte_solve_opts* o = c.o;
    GridView& gv = c.gv;
    PointParams& pp = c.pp;
    cudaStream_t s = c.s;
    int32_t* status = c.status;
    int32_t* iters = c.iters;
    const double wsz = (prec == BTE_PREC_MIXED) ? 4.0 : 8.0;
    const int nrefine = (prec == BTE_PREC_MIXED) ? std::min(std::max(o->refine, 0), 8) : 0;
    // a mixed-form point that needs more than 13 halvings goes to the FP64 path instead
    const double amin = (prec == BTE_PREC_MIXED) ? std::max(o->alpha_min, 1.0 / 8192.0) : o->alpha_min;
    Profiler& pf = g_prof;
    auto other = [&](auto&& fn) { return pf.run(PF_OTHER, s, 0, 0, 1, fn); };
    // points that switched to the double-double residual: their state's F, aux and merit again
    CKR(pf.run(PF_RESIDUAL, s, 0, 0, 2, [&] {
        k_residual<<<nact, 256, res_smem, s>>>(gv, pp, ee, L.act, nact, w->h, nullptr, 0, nullptr, w->ddpend, nullptr,
                                               w->F, w->aux, w->scal, w->r, nullptr, w->ddm);
        k_set_list<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, w->ddpend, 0);
    }));
    {
        // Jacobian straight into the factorization buffer, then LU of [J | -F] and back substitution
        dim3 gj(nblk(N, JAC_WARPS), nact);
        const double jb = (double)nact * N * (N + 1) * wsz;
        const double lub = 2.0 * (double)nact * N * (N + 1) * wsz;
        const double lsb = (double)nact * (0.5 * N * (N + 1) * wsz + N * wsz);
        cudaError_t le = cudaSuccess;
        if (prec == BTE_PREC_MIXED) {
            float* xs = reinterpret_cast<float*>(L.xs);
            CKR(pf.run(PF_JACOBIAN, s, nact * jac_flops_pt(g, ee), jb, 1, [&] {
                const JacSmem jm = jac_smem<float>(g, ee);
                k_jacobian<float><<<gj, JAC_WARPS * 32, jm.bytes, s>>>(gv, pp, ee, L.act, nact, w->h, w->F, w->aux, w->scal,
                                                                 (float*)L.J, ld, jstride, beta_scale, L.rowscale,
                                                                 jm.stage, 1.0, 0.0, L.kc);
            }));
            CKR(pf.run(PF_LU, s, nact * lu_flops(N), lub, 1, [&] {
                le = bte_lu_factor_t<float>(nact, N, N + 1, (float*)L.J, ld, jstride, L.piv, L.info, s,
                                            lu_kernel_for(o->lu_kernel, N));
            }));
            CKR(le);
            CKR(pf.run(PF_LUSOLVE, s, nact * (double)N * N, lsb, 1, [&] {
                le = bte_lu_solve_t<float>(nact, N, (const float*)L.J, ld, jstride, L.piv, xs, 1, s);
            }));
            CKR(le);
            CKR(other([&] { k_store_solution<float><<<nact, 128, 0, s>>>(nact, xs, N, L.act, w->dh, ldd); }));
            // FP64 iterative refinement of the step against the matrix-free FP64 Jacobian,
            // per point until its correction contracts (or it is handed to FP64)
            if (nrefine > 0) CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->refdone, 0, P); }));
            for (int rf = 0; rf < nrefine; ++rf) {
                double* cprev = (rf & 1) ? w->corr0 : w->corr1;
                double* ccur = (rf & 1) ? w->corr1 : w->corr0;
                CKR(pf.run(PF_REFINE, s, nact * (res_flops_pt(g, ee) + 2.0 * (double)N * N),
                           nact * (res_bytes_pt(g, true) + 0.5 * N * (N + 1) * wsz), 3, [&] {
                    k_refine_residual<<<nact, 256, ref_smem, s>>>(gv, pp, ee, L.act, nact, w->h, w->F, w->aux,
                                                                  w->scal, w->dh, ldd, beta_scale, L.rowscale, xs,
                                                                  L.sigma, w->refdone, L.kc, nullptr, 0, nullptr, 0,
                                                                  nullptr);
                    le = bte_lu_solve_t<float>(nact, N, (const float*)L.J, ld, jstride, L.piv, xs, 0, s);
                    k_refine_update<<<nact, 128, 0, s>>>(nact, L.act, N, xs, L.sigma, w->dh, ldd, ccur,
                                                         w->refdone);
                }));
                CKR(le);
                if (rf == 0)
                    CKR(other([&] { k_refine_first<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, ccur, w->refdone, 1e-5); }));
                if (rf >= 1)
                    CKR(other([&] {
                        k_refine_check<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, cprev, ccur, status, w->refdone,
                                                                       rf + 1 == nrefine);
                    }));
            }
            // points whose refinement stalled: GMRES on the same FP32 factors before any FP64 hand-over
            if (nrefine > 0 && w->gm_cap > 0 && o->krylov >= 0 && (o->krylov > 0 || N >= GM_MIN_N))
                CKR(gmres_refine(c, L, nact, o->krylov == 2));
        } else {
            double* xs = L.xs;
            CKR(pf.run(PF_JACOBIAN, s, nact * jac_flops_pt(g, ee), jb, 1, [&] {
                const JacSmem jm = jac_smem<double>(g, ee);
                k_jacobian<double><<<gj, JAC_WARPS * 32, jm.bytes, s>>>(gv, pp, ee, L.act, nact, w->h, w->F, w->aux, w->scal,
                                                                  (double*)L.J, ld, jstride, beta_scale, L.rowscale,
                                                                  jm.stage, 1.0, 0.0, nullptr);
            }));
            CKR(pf.run(PF_LU64, s, nact * lu_flops(N), lub, 1, [&] {
                le = bte_lu_factor_t<double>(nact, N, N + 1, (double*)L.J, ld, jstride, L.piv, L.info, s,
                                             lu64_kernel_for(o->lu64_kernel));
            }));
            CKR(le);
            CKR(pf.run(PF_LUSOLVE, s, nact * (double)N * N, lsb, 1, [&] {
                le = bte_lu_solve_t<double>(nact, N, (const double*)L.J, ld, jstride, L.piv, xs, 1, s);
            }));
            CKR(le);
            CKR(other([&] { k_store_solution<double><<<nact, 128, 0, s>>>(nact, xs, N, L.act, w->dh, ldd); }));
        }
        // per-point Armijo backtracking
        CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->searching, 0, P); }));
        CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->accepted, 0, P); }));
        CKR(other([&] { k_set_active<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, w->searching, w->alpha); }));
        int nsearch = nact;
        for (int ls = 0; ls < 200; ++ls) {
            CKR(pf.run(PF_RESIDUAL, s, nsearch * res_flops_pt(g, ee), nsearch * res_bytes_pt(g, true), 1, [&] {
                k_residual<<<nact, 256, res_smem, s>>>(gv, pp, ee, L.act, nact, w->h, w->dh, ldd, w->alpha,
                                                       w->searching, w->ht, w->Ft, w->auxt, w->scalt, w->rt, w->srel,
                                                       w->ddm);
            }));
            CKR(cudaMemsetAsync(w->cnt, 0, sizeof(int32_t), s));
            CKR(other([&] {
                k_armijo<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, w->searching, w->alpha, w->r, w->rt,
                                                        o->line_search_c, o->alpha_rho, amin, status, w->cnt,
                                                        w->accepted, w->r0, 1e-9, w->srel, 1e-8,
                                                        prec == BTE_PREC_MIXED ? BTE_ST_NEED_FP64 : BTE_ST_ROUNDOFF,
                                                        w->ddm, w->ddpend);
            }));
            int hc = 0;
            CKR(cudaMemcpyAsync(&hc, w->cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            CKR(cudaStreamSynchronize(s));
            nsearch = hc;
            if (hc == 0) break;
        }
        CKR(other([&] {
            k_accept<<<nact, 256, 0, s>>>(n, nact, L.act, w->accepted, w->h, w->ht, w->F, w->Ft, w->aux, w->auxt,
                                         w->scal, w->scalt, w->r, w->rt, iters);
        }));
        CKR(cudaMemsetAsync(w->cnt, 0, sizeof(int32_t), s));
        CKR(other([&] {
            k_converge<<<nblk(nact, 256), 256, 0, s>>>(nact, L.act, w->r, w->r0, o->atol, o->rtol,
                                                      w->nit, o->max_iter,
                                                      prec == BTE_PREC_MIXED ? MIXED_HANDOVER_ITER : 0, status, L.act2,
                                                      w->cnt, L.info, 0);
        }));
        int hn = 0;
        CKR(cudaMemcpyAsync(&hn, w->cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CKR(cudaStreamSynchronize(s));
        pf.drain(s);
        std::swap(L.act, L.act2);
        nact = hn;
    }
    return nact;
}

int bte_solve_impl(BteGrid* g, int P, const double* n0, const double* ne, const double* ns_by_n0, const double* Tg,
                   const double* E, double* f, int32_t* status, int32_t* iters, const bte_solve_opts* o,
                   cudaStream_t s) {
    if (P <= 0) return BTE_OK;
    BteWork* w = bte_work_get(g);
    const int prec = o->precision;
    int rc = ensure_work(w, g, P, prec, o->krylov);
    if (rc) return rc;
    SolveCtx c{};
    c.g = g; c.w = w; c.gv = view_of(g); c.pp = PointParams{n0, ne, Tg, E, ns_by_n0, P};
    c.P = P; c.n = g->n; c.N = g->n + 1; c.ld = (c.N + 1 + 3) & ~3; c.ldd = c.N + 1;
    c.ee = (o->ee && g->ee) ? 1 : 0;
    c.jstride = (long long)c.N * c.ld;
    // border scale: typical magnitude of the raw collision operator per unit n0
    c.beta_scale = g->q0max / (g->umax > 0 ? g->umax : 1.0);
    c.res_smem = (size_t)7 * c.n * sizeof(double);
    c.ref_smem = (size_t)(5 * c.n + 2) * sizeof(double);  // x, r: n + 1 each; h, HL x, GL x: n each
    c.o = o; c.status = status; c.iters = iters; c.s = s;
    const int n = c.n;
    CKR(bte_raise_smem_limit((const void*)k_residual, c.res_smem));
    CKR(bte_raise_smem_limit((const void*)k_refine_residual, c.ref_smem));
    Profiler& pf = g_prof;
    Lane L{w->act, w->act2, w->J, w->piv, w->info, w->xs, w->rowscale, w->sigma, w->kc};
    auto other = [&](auto&& fn) { return pf.run(PF_OTHER, s, 0, 0, 1, fn); };
    auto residual_all = [&](int nact) {
        return pf.run(PF_RESIDUAL, s, nact * res_flops_pt(g, c.ee), nact * res_bytes_pt(g, false), 1, [&] {
            k_residual<<<nact, 256, c.res_smem, s>>>(c.gv, c.pp, c.ee, L.act, nact, w->h, nullptr, 0, nullptr,
                                                     nullptr, nullptr, w->F, w->aux, w->scal, w->r, nullptr, w->ddm);
        });
    };

    CKR(other([&] { k_mass_normalize<<<P, 256, 0, s>>>(n, g->d_u, f, w->h, P); }));
    CKR(cudaMemcpyAsync(w->h0, w->h, (size_t)P * n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(status, -1, P); }));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(iters, 0, P); }));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->nit, 0, P); }));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->ddm, 0, P); }));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->ddpend, 0, P); }));
    CKR(other([&] { k_iota<<<nblk(P, 256), 256, 0, s>>>(L.act, P); }));
    CKR(residual_all(P));
    CKR(cudaMemcpyAsync(w->r0, w->r, P * sizeof(double), cudaMemcpyDeviceToDevice, s));
    const size_t rm_smem = (size_t)2 * n * sizeof(double);
    CKR(bte_raise_smem_limit((const void*)k_ref_merit, rm_smem));
    CKR(other([&] { k_ref_merit<<<P, 256, rm_smem, s>>>(c.gv, P, nullptr, w->F, w->ref_r0); }));
    for (int it = 0, nact = P; it < o->max_iter && nact > 0; ++it) {
        nact = newton_iteration(c, L, nact, prec);
        if (nact < 0) return nact;
    }
    if (prec == BTE_PREC_MIXED) {
        // points the mixed form did not converge go to the FP64 form (k_restore: from where)
        CKR(cudaMemsetAsync(w->cnt, 0, sizeof(int32_t), s));
        CKR(other([&] { k_collect_failed<<<nblk(P, 256), 256, 0, s>>>(P, status, L.act2, w->cnt, w->reason); }));
        int nf = 0;
        CKR(cudaMemcpyAsync(&nf, w->cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CKR(cudaStreamSynchronize(s));
        // FP64 chunks of as many matrices as the J buffer holds in FP64 (at least one)
        const int chunk = (int)std::min<size_t>((size_t)P, w->jbytes / ((size_t)c.N * c.ld * sizeof(double)));
        if (chunk < 1) return BTE_ERR_STATE;
        std::vector<int32_t> failed(nf);
        if (nf) CKR(cudaMemcpyAsync(failed.data(), L.act2, nf * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CKR(cudaStreamSynchronize(s));
        long long why[8] = {0};
        if (nf && pf.on) {  // why they failed (statuses were reset to running by k_collect_failed)
            std::vector<int32_t> st(P);
            CKR(cudaMemcpy(st.data(), w->reason, P * sizeof(int32_t), cudaMemcpyDeviceToHost));
            for (int i = 0; i < nf; ++i) {
                int r = st[failed[i]];
                if (r >= 0 && r < 8) why[r]++;
            }
        }
        pf.count_fallback(nf, why);
        for (int c0 = 0; c0 < nf; c0 += chunk) {
            int m = std::min(chunk, nf - c0);
            CKR(cudaMemcpyAsync(L.act, failed.data() + c0, m * sizeof(int32_t), cudaMemcpyHostToDevice, s));
            CKR(other([&] { k_restore<<<m, 256, 0, s>>>(n, m, L.act, w->reason, w->h0, w->h, w->nit, w->r, w->r0); }));
            CKR(other([&] { k_set_list<<<nblk(m, 256), 256, 0, s>>>(m, L.act, w->ddm, 0); }));
            CKR(residual_all(m));
            for (int it = 0, nact = m; it < o->max_iter && nact > 0; ++it) {
                nact = newton_iteration(c, L, nact, BTE_PREC_FP64);
                if (nact < 0) return nact;
            }
        }
    }
    const double c_gamma = std::sqrt(2.0 * (BTE_QE / BTE_ME));
    const double mm_fac = std::sqrt(1.0 / (4.0 * M_PI)) * 4.0 * M_PI;
    const double sc3 = 2.0 * std::pow(g->vth / c_gamma, 3);
    CKR(other([&] { k_normalized_distribution<<<P, 256, 0, s>>>(n, g->d_mass, mm_fac, sc3, w->h, f, P); }));
    CKR(other([&] { k_ref_merit<<<P, 256, rm_smem, s>>>(c.gv, P, nullptr, w->F, w->ref_r); }));
    return BTE_OK;
}

// per-point residual norms of the last steady solve on this grid: r_final, r_initial
int bte_solve_info_impl(BteGrid* g, int P, double* r_final, double* r_initial, cudaStream_t s) {
    BteWork* w = g->work;
    if (!w || w->cap < P) return BTE_ERR_STATE;
    if (cudaMemcpyAsync(r_final, w->ref_r, P * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return BTE_ERR_CUDA;
    if (cudaMemcpyAsync(r_initial, w->ref_r0, P * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return BTE_ERR_CUDA;
    return BTE_OK;
}

// ---------------------------------------------------------------------------------
// Serving engine: a fixed set of point slots on one grid, resident on the device. Points
// enter free slots between Newton iterations and leave as soon as their own solve ends, so
// requests that arrive while others run join the same launches (continuous batching at the
// granularity of one Newton iteration). Each slot runs the reference driver's two solves
// (bte_0d3v_batched_driver.py:192-204): phase 0 without e-e collisions from the admitted
// state, then, if the request asks for e-e, phase 1 with them from phase 0's normalized
// result. Per point the arithmetic is that of bte_solve_steady: in the mixed form a point
// whose FP32 solve fails moves to an FP64 lane (its own Jacobian buffers, fcap slots) for
// the rest of that phase, from the same state bte_solve_steady would use.
// ---------------------------------------------------------------------------------
struct BteEngine {
    BteGrid* g = nullptr;
    int cap = 0, fcap = 0, prec = 0;
    bte_solve_opts opts{};
    BteWork w;          // per-slot state; its position-indexed buffers serve the main lane
    Lane main{}, f64{}; // f64: mixed form only
    void* J64 = nullptr;
    int32_t *piv64 = nullptr, *info64 = nullptr, *act64a = nullptr, *act64b = nullptr;
    double *xs64 = nullptr, *rs64 = nullptr, *sg64 = nullptr;
    double *n0 = nullptr, *ne = nullptr, *Tg = nullptr, *E = nullptr, *ns = nullptr;  // per slot, ns species-major
    int8_t *phase = nullptr, *want_ee = nullptr;   // per slot
    int32_t *status = nullptr, *iters = nullptr;   // per slot
    int32_t *l_done = nullptr, *l_fb = nullptr, *l_sw = nullptr, *l_in = nullptr, *cnt = nullptr;
    int nmain = 0, nf64 = 0;
    std::vector<int> free_slots;
    std::deque<int> f64_wait;   // slots waiting for room in the FP64 lane
    std::vector<void*> allocs;
    size_t bytes = 0;           // device memory held
};

__global__ void k_engine_admit(int m, const int* __restrict__ slots, int n, const double* __restrict__ u,
                               const double* __restrict__ f0, double* h, double* h0, const double* __restrict__ n0_in,
                               const double* __restrict__ ne_in, const double* __restrict__ Tg_in,
                               const double* __restrict__ E_in, const double* __restrict__ ns_in, int nspecies,
                               double* n0, double* ne, double* Tg, double* E, double* ns, int cap, int8_t* phase,
                               int8_t* want_ee, int want, int* status, int* iters, int* nit) {
    __shared__ double red[32];
    const int i = blockIdx.x;
    if (i >= m) return;
    const int pt = slots[i];
    // the state enters as bte_solve_steady takes it: h = f0 / (u . f0)
    double sacc = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) sacc += u[k] * f0[(size_t)i * n + k];
    sacc = block_sum(sacc, red);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double v = f0[(size_t)i * n + k] / sacc;
        h[(size_t)pt * n + k] = v;
        h0[(size_t)pt * n + k] = v;
    }
    if (threadIdx.x == 0) {
        n0[pt] = n0_in[i]; ne[pt] = ne_in[i]; Tg[pt] = Tg_in[i]; E[pt] = E_in[i];
        for (int sp = 0; sp < nspecies; ++sp) ns[(size_t)sp * cap + pt] = ns_in[(size_t)sp * m + i];
        phase[pt] = 0; want_ee[pt] = (int8_t)want; status[pt] = -1; iters[pt] = 0; nit[pt] = 0;
    }
}

__global__ void k_copy_list(int m, const int* __restrict__ list, const double* __restrict__ src, double* dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) dst[list[i]] = src[list[i]];
}

// sort the points that left a lane in its last iteration: finished (done), handed to the FP64
// lane (fb, mixed main lane only), or switching to the e-e phase (sw)
__global__ void k_engine_sort(int nold, const int* __restrict__ old, const int* __restrict__ status,
                              const int8_t* __restrict__ phase, const int8_t* __restrict__ want_ee, int can_fb,
                              int* done, int* fb, int* sw, int* cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nold) return;
    const int pt = old[i];
    const int st = status[pt];
    if (st < 0) return;  // still running
    if (can_fb && st >= BTE_ST_LINESEARCH) { fb[atomicAdd(&cnt[1], 1)] = pt; return; }
    if (st <= BTE_ST_ROUNDOFF && phase[pt] == 0 && want_ee[pt]) { sw[atomicAdd(&cnt[2], 1)] = pt; return; }
    done[atomicAdd(&cnt[0], 1)] = pt;
}

// a point entering the FP64 lane: as k_collect_failed + k_restore do in bte_solve_steady
__global__ void k_engine_to_fp64(int m, const int* __restrict__ list, int n, int* status, int* reason, int* nit,
                                 const double* __restrict__ h0, double* h, const double* __restrict__ r,
                                 const double* __restrict__ r0) {
    const int i = blockIdx.x;
    if (i >= m) return;
    const int pt = list[i];
    const int st = status[pt];
    __syncthreads();
    if (threadIdx.x == 0) { reason[pt] = st; status[pt] = -1; }
    if (!handover_restarts(st, nit[pt], r[pt], r0[pt])) return;
    for (int k = threadIdx.x; k < n; k += blockDim.x) h[(size_t)pt * n + k] = h0[(size_t)pt * n + k];
}

// phase 0 -> phase 1: the state bte_solve_steady's second call starts from, i.e. the
// normalized distribution of the first call, mass-normalized again
__global__ void k_engine_phase1(int m, const int* __restrict__ list, int n, const double* __restrict__ mass,
                                double mm_fac, double scale3, const double* __restrict__ u, double* h, double* h0,
                                int8_t* phase, int* status, int* nit) {
    __shared__ double red[32];
    const int i = blockIdx.x;
    if (i >= m) return;
    const int pt = list[i];
    double* hp = h + (size_t)pt * n;
    double sacc = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) sacc += (mass[k] / mm_fac) * hp[k];
    sacc = block_sum(sacc, red) * scale3;
    for (int k = threadIdx.x; k < n; k += blockDim.x) hp[k] = hp[k] / sacc;
    double s2 = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) s2 += u[k] * hp[k];
    s2 = block_sum(s2, red);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double v = hp[k] / s2;
        hp[k] = v;
        h0[(size_t)pt * n + k] = v;
    }
    if (threadIdx.x == 0) { phase[pt] = 1; status[pt] = -1; nit[pt] = 0; }
}

__global__ void k_engine_collect(int m, const int* __restrict__ list, int n, const double* __restrict__ mass,
                                 double mm_fac, double scale3, const double* __restrict__ h,
                                 const int* __restrict__ status, const int* __restrict__ iters, double* f,
                                 int32_t* st_out, int32_t* it_out) {
    __shared__ double red[32];
    const int i = blockIdx.x;
    if (i >= m) return;
    const int pt = list[i];
    const double* hp = h + (size_t)pt * n;
    double sacc = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) sacc += (mass[k] / mm_fac) * hp[k];
    sacc = block_sum(sacc, red) * scale3;
    for (int k = threadIdx.x; k < n; k += blockDim.x) f[(size_t)i * n + k] = hp[k] / sacc;
    if (threadIdx.x == 0) {
        if (st_out) st_out[i] = status[pt];
        if (it_out) it_out[i] = iters[pt];
    }
}

static void engine_free(BteEngine* e) {
    for (void* p : e->allocs) cudaFree(p);
    e->allocs.clear();
    free_work(&e->w);
}

static SolveCtx engine_ctx(BteEngine* e, cudaStream_t s) {
    BteGrid* g = e->g;
    SolveCtx c{};
    c.g = g; c.w = &e->w; c.gv = view_of(g);
    c.pp = PointParams{e->n0, e->ne, e->Tg, e->E, e->ns, e->cap, e->phase};
    c.P = e->cap; c.n = g->n; c.N = g->n + 1; c.ld = (c.N + 1 + 3) & ~3; c.ldd = c.N + 1;
    c.ee = g->ee ? 1 : 0;  // per point: the slot's phase
    c.jstride = (long long)c.N * c.ld;
    c.beta_scale = g->q0max / (g->umax > 0 ? g->umax : 1.0);
    c.res_smem = (size_t)7 * c.n * sizeof(double);
    c.ref_smem = (size_t)(5 * c.n + 2) * sizeof(double);  // x, r: n + 1 each; h, HL x, GL x: n each
    c.o = &e->opts; c.status = e->status; c.iters = e->iters; c.s = s;
    return c;
}

int bte_engine_create_impl(BteGrid* g, int cap, int fcap, const bte_solve_opts* o, BteEngine** out) {
    BteEngine* e = new BteEngine();
    e->g = g; e->cap = cap; e->prec = o->precision; e->opts = *o;
    e->fcap = (o->precision == BTE_PREC_MIXED) ? std::max(1, std::min(fcap, cap)) : 0;
    const int n = g->n, N = n + 1, ld = (N + 1 + 3) & ~3;
    int rc = ensure_work(&e->w, g, cap, e->prec, o->krylov);
    if (rc) { delete e; return rc; }
    e->bytes = e->w.jbytes + e->w.kcbytes + e->w.gmbytes + (size_t)cap * (size_t)(n * 12 + (N + 1) * 3 + 24) * sizeof(double);  // J + per-slot vectors
    bool ok = true;
    auto A = [&](void** p, size_t bytes) {
        if (!ok) return;
        if (cudaMalloc(p, std::max<size_t>(bytes, 8)) != cudaSuccess) { ok = false; *p = nullptr; return; }
        e->allocs.push_back(*p);
        e->bytes += bytes;
    };
    const size_t dc = (size_t)cap * sizeof(double), ic = (size_t)cap * sizeof(int32_t);
    A((void**)&e->n0, dc); A((void**)&e->ne, dc); A((void**)&e->Tg, dc); A((void**)&e->E, dc);
    A((void**)&e->ns, dc * g->nspecies);
    A((void**)&e->phase, cap); A((void**)&e->want_ee, cap);
    A((void**)&e->status, ic); A((void**)&e->iters, ic);
    A((void**)&e->l_done, ic); A((void**)&e->l_fb, ic); A((void**)&e->l_sw, ic); A((void**)&e->l_in, ic);
    A((void**)&e->cnt, 4 * sizeof(int32_t));
    if (e->fcap > 0) {
        const int f = e->fcap;
        A(&e->J64, (size_t)f * N * ld * sizeof(double));
        A((void**)&e->piv64, (size_t)f * N * sizeof(int32_t)); A((void**)&e->info64, (size_t)f * sizeof(int32_t));
        A((void**)&e->act64a, (size_t)f * sizeof(int32_t)); A((void**)&e->act64b, (size_t)f * sizeof(int32_t));
        A((void**)&e->xs64, (size_t)f * (N + 1) * sizeof(double)); A((void**)&e->rs64, (size_t)f * (N + 1) * sizeof(double));
        A((void**)&e->sg64, (size_t)f * sizeof(double));
    }
    if (!ok) { engine_free(e); delete e; return BTE_ERR_ALLOC; }
    e->main = Lane{e->w.act, e->w.act2, e->w.J, e->w.piv, e->w.info, e->w.xs, e->w.rowscale, e->w.sigma, e->w.kc};
    e->f64 = Lane{e->act64a, e->act64b, e->J64, e->piv64, e->info64, e->xs64, e->rs64, e->sg64, nullptr};
    e->free_slots.resize(cap);
    for (int i = 0; i < cap; ++i) e->free_slots[i] = cap - 1 - i;  // pop_back hands out 0, 1, 2, ...
    SolveCtx c = engine_ctx(e, 0);
    if (bte_raise_smem_limit((const void*)k_residual, c.res_smem) != cudaSuccess) { engine_free(e); delete e; return BTE_ERR_CUDA; }
    if (bte_raise_smem_limit((const void*)k_refine_residual, c.ref_smem) != cudaSuccess) { engine_free(e); delete e; return BTE_ERR_CUDA; }
    const size_t rm_smem = (size_t)2 * n * sizeof(double);
    if (bte_raise_smem_limit((const void*)k_ref_merit, rm_smem) != cudaSuccess) { engine_free(e); delete e; return BTE_ERR_CUDA; }
    *out = e;
    return BTE_OK;
}

void bte_engine_destroy_impl(BteEngine* e) {
    if (!e) return;
    engine_free(e);
    delete e;
}

int bte_engine_free_slots(const BteEngine* e) { return (int)e->free_slots.size(); }
int bte_engine_active(const BteEngine* e) { return e->nmain + e->nf64 + (int)e->f64_wait.size(); }
int bte_engine_fp64_capacity(const BteEngine* e) { return e->fcap; }
int bte_engine_capacity(const BteEngine* e) { return e->cap; }
BteGrid* bte_engine_grid(const BteEngine* e) { return e->g; }
size_t bte_engine_bytes(const BteEngine* e) { return e->bytes; }

// residual, r0 and the reference merit at the start of a phase, for the m slots in `list`
static int engine_start_phase(BteEngine* e, SolveCtx& c, const int* list, int m, cudaStream_t s) {
    if (m <= 0) return BTE_OK;
    BteGrid* g = e->g;
    BteWork* w = &e->w;
    const int n = g->n;
    Profiler& pf = g_prof;
    CKR(pf.run(PF_RESIDUAL, s, m * res_flops_pt(g, c.ee), m * res_bytes_pt(g, false), 1, [&] {
        k_residual<<<m, 256, c.res_smem, s>>>(c.gv, c.pp, c.ee, list, m, w->h, nullptr, 0, nullptr, nullptr, nullptr,
                                              w->F, w->aux, w->scal, w->r, nullptr, nullptr);
    }));
    CKR(pf.run(PF_OTHER, s, 0, 0, 4, [&] {
        k_set_list<<<nblk(m, 256), 256, 0, s>>>(m, list, w->ddm, 0);
        k_set_list<<<nblk(m, 256), 256, 0, s>>>(m, list, w->ddpend, 0);
        k_copy_list<<<nblk(m, 256), 256, 0, s>>>(m, list, w->r, w->r0);
        k_ref_merit<<<m, 256, (size_t)2 * n * sizeof(double), s>>>(c.gv, m, list, w->F, w->ref_r0);
    }));
    return BTE_OK;
}

int bte_engine_admit_impl(BteEngine* e, int m, const double* n0, const double* ne, const double* ns_by_n0,
                          const double* Tg, const double* E, const double* f0, int want_ee, int32_t* slots_out,
                          cudaStream_t s) {
    if (m <= 0) return BTE_OK;
    if (m > (int)e->free_slots.size()) return BTE_ERR_STATE;
    BteGrid* g = e->g;
    const int n = g->n;
    std::vector<int32_t> sl(m);
    for (int i = 0; i < m; ++i) { sl[i] = e->free_slots.back(); e->free_slots.pop_back(); }
    SolveCtx c = engine_ctx(e, s);
    Profiler& pf = g_prof;
    CKR(cudaMemcpyAsync(e->l_in, sl.data(), m * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    CKR(pf.run(PF_OTHER, s, 0, 0, 1, [&] {
        k_engine_admit<<<m, 256, 0, s>>>(m, e->l_in, n, g->d_u, f0, e->w.h, e->w.h0, n0, ne, Tg, E, ns_by_n0,
                                         g->nspecies, e->n0, e->ne, e->Tg, e->E, e->ns, e->cap, e->phase, e->want_ee,
                                         want_ee ? 1 : 0, e->status, e->iters, e->w.nit);
    }));
    int rc = engine_start_phase(e, c, e->l_in, m, s);
    if (rc) return rc;
    CKR(cudaMemcpyAsync(e->main.act + e->nmain, e->l_in, m * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    e->nmain += m;
    CKR(cudaStreamSynchronize(s));  // the host list `sl` and the slot order are settled
    for (int i = 0; i < m; ++i) slots_out[i] = sl[i];
    return BTE_OK;
}

int bte_engine_step_impl(BteEngine* e, int* n_done, int32_t* done_out, cudaStream_t s) {
    *n_done = 0;
    BteGrid* g = e->g;
    BteWork* w = &e->w;
    const int n = g->n;
    SolveCtx c = engine_ctx(e, s);
    Profiler& pf = g_prof;
    const bool mixed = (e->prec == BTE_PREC_MIXED);
    // points waiting for the FP64 lane move in while it has room
    const int room = e->fcap - e->nf64;
    const int k = std::min<int>(room, (int)e->f64_wait.size());
    if (mixed && k > 0) {
        std::vector<int32_t> mv(k);
        for (int i = 0; i < k; ++i) { mv[i] = e->f64_wait.front(); e->f64_wait.pop_front(); }
        CKR(cudaMemcpyAsync(e->l_in, mv.data(), k * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        CKR(pf.run(PF_OTHER, s, 0, 0, 1, [&] {
            k_engine_to_fp64<<<k, 256, 0, s>>>(k, e->l_in, n, e->status, w->reason, w->nit, w->h0, w->h, w->r, w->r0);
        }));
        CKR(pf.run(PF_RESIDUAL, s, k * res_flops_pt(g, c.ee), k * res_bytes_pt(g, false), 1, [&] {
            k_set_list<<<nblk(k, 256), 256, 0, s>>>(k, e->l_in, w->ddm, 0);
            k_residual<<<k, 256, c.res_smem, s>>>(c.gv, c.pp, c.ee, e->l_in, k, w->h, nullptr, 0, nullptr, nullptr,
                                                  nullptr, w->F, w->aux, w->scal, w->r, nullptr, nullptr);
        }));
        CKR(cudaMemcpyAsync(e->f64.act + e->nf64, e->l_in, k * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        CKR(cudaStreamSynchronize(s));  // `mv` is read by the copy above
        e->nf64 += k;
    }
    CKR(cudaMemsetAsync(e->cnt, 0, 4 * sizeof(int32_t), s));
    if (e->nmain > 0) {
        const int nold = e->nmain;
        const int r = newton_iteration(c, e->main, nold, e->prec);
        if (r < 0) return r;
        e->nmain = r;
        CKR(pf.run(PF_OTHER, s, 0, 0, 1, [&] {
            k_engine_sort<<<nblk(nold, 256), 256, 0, s>>>(nold, e->main.act2, e->status, e->phase, e->want_ee,
                                                          mixed ? 1 : 0, e->l_done, e->l_fb, e->l_sw, e->cnt);
        }));
    }
    if (e->nf64 > 0) {
        const int nold = e->nf64;
        const int r = newton_iteration(c, e->f64, nold, BTE_PREC_FP64);
        if (r < 0) return r;
        e->nf64 = r;
        CKR(pf.run(PF_OTHER, s, 0, 0, 1, [&] {
            k_engine_sort<<<nblk(nold, 256), 256, 0, s>>>(nold, e->f64.act2, e->status, e->phase, e->want_ee, 0,
                                                          e->l_done, e->l_fb, e->l_sw, e->cnt);
        }));
    }
    int hc[4] = {0, 0, 0, 0};
    CKR(cudaMemcpyAsync(hc, e->cnt, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CKR(cudaStreamSynchronize(s));
    const int nd = hc[0], nfb = hc[1], nsw = hc[2];
    if (nfb > 0) {
        std::vector<int32_t> fb(nfb);
        CKR(cudaMemcpyAsync(fb.data(), e->l_fb, nfb * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CKR(cudaStreamSynchronize(s));
        for (int v : fb) e->f64_wait.push_back(v);
        pf.count_fallback(nfb, nullptr);
    }
    if (nsw > 0) {
        const double c_gamma = std::sqrt(2.0 * (BTE_QE / BTE_ME));
        const double mm_fac = std::sqrt(1.0 / (4.0 * M_PI)) * 4.0 * M_PI;
        const double sc3 = 2.0 * std::pow(g->vth / c_gamma, 3);
        CKR(pf.run(PF_OTHER, s, 0, 0, 1, [&] {
            k_engine_phase1<<<nsw, 256, 0, s>>>(nsw, e->l_sw, n, g->d_mass, mm_fac, sc3, g->d_u, w->h, w->h0,
                                                e->phase, e->status, w->nit);
        }));
        int rc = engine_start_phase(e, c, e->l_sw, nsw, s);
        if (rc) return rc;
        CKR(cudaMemcpyAsync(e->main.act + e->nmain, e->l_sw, nsw * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        e->nmain += nsw;
    }
    if (nd > 0) CKR(cudaMemcpyAsync(done_out, e->l_done, nd * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CKR(cudaStreamSynchronize(s));
    *n_done = nd;
    return BTE_OK;
}

int bte_engine_collect_impl(BteEngine* e, int m, const int32_t* slots, double* f, int32_t* status, int32_t* iters,
                            cudaStream_t s) {
    if (m <= 0) return BTE_OK;
    BteGrid* g = e->g;
    for (int i = 0; i < m; ++i)
        if (slots[i] < 0 || slots[i] >= e->cap) return BTE_ERR_ARG;
    CKR(cudaMemcpyAsync(e->l_in, slots, m * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    const double c_gamma = std::sqrt(2.0 * (BTE_QE / BTE_ME));
    const double mm_fac = std::sqrt(1.0 / (4.0 * M_PI)) * 4.0 * M_PI;
    const double sc3 = 2.0 * std::pow(g->vth / c_gamma, 3);
    CKR(g_prof.run(PF_OTHER, s, 0, 0, 1, [&] {
        k_engine_collect<<<m, 256, 0, s>>>(m, e->l_in, g->n, g->d_mass, mm_fac, sc3, e->w.h, e->status, e->iters, f,
                                           status, iters);
    }));
    CKR(cudaStreamSynchronize(s));
    for (int i = 0; i < m; ++i) e->free_slots.push_back(slots[i]);
    return BTE_OK;
}

// ---------------------------------------------------------------------------------
// Transient solve (solve(..., "transient"), bte_0d3v_batched.py:1063-1155, with
// newton_solver_batched, :59-126): backward Euler, t in RF periods, tau = 1 / efreq
// (1e-7 without a field frequency). Each step solves, for the increment delta with
// u . delta = 0 (the reference's du in the mass-conserving coordinates Q du),
//     M delta - dt tau F_raw(h + delta) - lambda M p = 0,
// by a chord iteration: the bordered Jacobian M - dt tau dF_raw/dh is built and factored once
// per step at the step's start state, as the reference inverts its Jacobian once per step,
// and reused for every iteration (no line search). A point's step ends when
// ||(I - p p^T) M^-1 G|| <= atol or <= rtol times its first value; the previous step's
// increment starts the next step's iteration, as in the reference. The cycle average of
// the state (trapezoid over each RF period) is kept for the QoIs.
// ---------------------------------------------------------------------------------
__global__ void k_add_iter(int P, const int* __restrict__ done, int* iters) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P && !done[i]) iters[i] += 1;
}

__global__ void k_set_efield(int P, const double* __restrict__ eRe, const double* __restrict__ eIm, double t,
                             const double* __restrict__ E0, int harmonic, double* E) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    E[i] = harmonic ? eRe[i] * cos(2.0 * BTE_PI * t) + eIm[i] * sin(2.0 * BTE_PI * t) : E0[i];
}

// G = M delta - c F  (M: the banded radial mass matrix, identical per harmonic)
__global__ void k_transient_G(GridView g, int nact, const int* __restrict__ act, const double* __restrict__ dh,
                              int ldd, const double* __restrict__ F, double c, double* G) {
    const int slot = blockIdx.x;
    if (slot >= nact) return;
    const int pt = act[slot];
    const int n = g.n, nsh = g.nsh, nsp = g.nsp;
    const double* d = dh + (size_t)pt * ldd;
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        const int p = a / nsh, q = a % nsh;
        double m = 0.0;
        for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
            const int k = p + dk;
            if (k >= 0 && k < nsp) m += g.Mr[p * BTE_NB + dk + BTE_BAND] * d[k * nsh + q];
        }
        G[(size_t)pt * n + a] = m - c * F[(size_t)pt * n + a];
    }
}

// points whose step converged leave the list; the others go on
__global__ void k_transient_conv(int nact, const int* __restrict__ act, const double* __restrict__ r,
                                 const double* __restrict__ r0, double atol, double rtol, int* done, int* act_out,
                                 int* nout) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nact) return;
    const int pt = act[i];
    const double rr = r[pt];
    if (rr <= atol || rr <= rtol * r0[pt]) { done[pt] = 1; return; }
    act_out[atomicAdd(nout, 1)] = pt;
}

// right-hand side of the chord step for every point (zero for points already done), row-scaled
// as the factored Jacobian: [-G; -beta u . delta]
template <typename T>
__global__ void k_transient_rhs(int P, int n, const double* __restrict__ G, const double* __restrict__ u,
                                const double* __restrict__ dh, int ldd, double beta, const double* __restrict__ rowscale,
                                const int* __restrict__ done, T* xs) {
    __shared__ double red[32];
    const int pt = blockIdx.x;
    if (pt >= P) return;
    const int N = n + 1;
    T* x = xs + (size_t)pt * N;
    if (done[pt]) {
        for (int a = threadIdx.x; a < N; a += blockDim.x) x[a] = T(0);
        return;
    }
    const double* d = dh + (size_t)pt * ldd;
    const double* rs = rowscale + (size_t)pt * N;
    double ud = 0.0;
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        x[a] = (T)(-G[(size_t)pt * n + a] * rs[a]);
        ud += u[a] * d[a];
    }
    ud = block_sum(ud, red);
    if (threadIdx.x == 0) x[n] = (T)(-beta * ud * rs[n]);
}

template <typename T>
__global__ void k_transient_update(int P, int n, const int* __restrict__ done, const T* __restrict__ xs, double* dh,
                                   int ldd) {
    const int pt = blockIdx.x;
    if (pt >= P || done[pt]) return;
    for (int a = threadIdx.x; a < n; a += blockDim.x) dh[(size_t)pt * ldd + a] += (double)xs[(size_t)pt * (n + 1) + a];
}

// avg += h (the trapezoid sums of the cycle average)
__global__ void k_accumulate(size_t m, const double* __restrict__ h, double* avg) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) avg[i] += h[i];
}
// h += delta (state update)
__global__ void k_apply_increment(int P, int n, const double* __restrict__ dh, int ldd, double* h) {
    const int pt = blockIdx.x;
    if (pt >= P) return;
    for (int a = threadIdx.x; a < n; a += blockDim.x) h[(size_t)pt * n + a] += dh[(size_t)pt * ldd + a];
}
__global__ void k_scale_into(size_t m, double c, double* a, double* b) {  // b = c a, a = 0
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) { b[i] = c * a[i]; a[i] = 0.0; }
}

int bte_transient_impl(BteGrid* g, int P, const double* n0, const double* ne, const double* ns_by_n0,
                       const double* Tg, const double* E, const double* eRe, const double* eIm, double* f,
                       double* f_avg, int32_t* status, int32_t* iters, const bte_transient_opts* o, cudaStream_t s) {
    if (P <= 0) return BTE_OK;
    BteWork* w = bte_work_get(g);
    // the step Jacobian M - dt tau dF/dh carries the B-spline mass matrix's conditioning
    // (1e5 and more at the configs' grids) on top of the step's own; FP32 factors do not
    // resolve it, so both forms factor it in FP64
    const int prec = BTE_PREC_FP64;
    int rc = ensure_work(w, g, P, prec);
    if (rc) return rc;
    const int n = g->n, N = n + 1;
    double *Et = nullptr, *avg = nullptr, *avgv = nullptr, *G = nullptr;
    int32_t* all = nullptr;
    CKR(cudaMallocAsync((void**)&all, (size_t)P * sizeof(int32_t), s));
    CKR(cudaMallocAsync((void**)&Et, (size_t)P * sizeof(double), s));
    CKR(cudaMallocAsync((void**)&avg, (size_t)P * n * sizeof(double), s));
    CKR(cudaMallocAsync((void**)&avgv, (size_t)P * n * sizeof(double), s));
    CKR(cudaMallocAsync((void**)&G, (size_t)P * n * sizeof(double), s));
    bte_solve_opts so{};
    so.atol = o->atol; so.rtol = o->rtol; so.max_iter = o->max_iter; so.ee = o->ee; so.precision = prec;
    SolveCtx c{};
    c.g = g; c.w = w; c.gv = view_of(g); c.pp = PointParams{n0, ne, Tg, Et, ns_by_n0, P, nullptr};
    c.P = P; c.n = n; c.N = N; c.ld = (N + 1 + 3) & ~3; c.ldd = N + 1;
    c.ee = (o->ee && g->ee) ? 1 : 0;
    c.jstride = (long long)N * c.ld;
    c.beta_scale = g->q0max / (g->umax > 0 ? g->umax : 1.0);
    c.res_smem = (size_t)7 * n * sizeof(double);
    c.o = &so; c.status = status; c.iters = iters; c.s = s;
    CKR(bte_raise_smem_limit((const void*)k_residual, c.res_smem));
    const size_t rm_smem = (size_t)2 * n * sizeof(double);
    CKR(bte_raise_smem_limit((const void*)k_ref_merit, rm_smem));
    Profiler& pf = g_prof;
    auto other = [&](auto&& fn) { return pf.run(PF_OTHER, s, 0, 0, 1, fn); };
    const int harmonic = o->efreq > 0 ? 1 : 0;
    const double tau = harmonic ? 1.0 / o->efreq : 1e-7;
    const double cdt = o->dt * tau;
    const int steps_total = (int)(o->cycles / o->dt);
    const int io_freq = std::max(1, (int)(1.0 / o->dt));
    const int ld = c.ld, ldd = c.ldd;
    const long long js = c.jstride;
    // border scale of the backward-Euler matrix: the mass matrix's magnitude over u's
    std::vector<double> mr((size_t)g->nsp * BTE_NB);
    CKR(cudaMemcpy(mr.data(), g->d_Mr, mr.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double mmax = 0.0;
    for (double v : mr) mmax = std::max(mmax, std::fabs(v));
    const double beta = mmax / (g->umax > 0 ? g->umax : 1.0);
    // state h = f / (u . f), increment 0, cycle sums 0
    CKR(other([&] { k_mass_normalize<<<P, 256, 0, s>>>(n, g->d_u, f, w->h, P); }));
    CKR(cudaMemsetAsync(w->dh, 0, (size_t)P * ldd * sizeof(double), s));
    CKR(cudaMemsetAsync(avg, 0, (size_t)P * n * sizeof(double), s));
    CKR(cudaMemsetAsync(avgv, 0, (size_t)P * n * sizeof(double), s));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(status, 0, P); }));
    CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(iters, 0, P); }));
    CKR(other([&] { k_fill_dbl<<<nblk(P, 256), 256, 0, s>>>(w->alpha, 1.0, P); }));
    CKR(other([&] { k_iota<<<nblk(P, 256), 256, 0, s>>>(all, P); }));
    double t = 0.0;
    int failed = 0;
    for (int ts = 0; ts <= steps_total; ++ts) {
        if (ts > 0 && ts % io_freq == 0 && ts == steps_total) {
            // the reference computes this last step but stops before applying it
            CKR(other([&] { k_scale_into<<<nblk(P * n, 256), 256, 0, s>>>((size_t)P * n, 0.5 * o->dt, avg, avgv); }));
            break;
        }
        CKR(other([&] { k_set_efield<<<nblk(P, 256), 256, 0, s>>>(P, eRe, eIm, t + o->dt, E, harmonic, Et); }));
        // the step's Jacobian at the current state, factored once
        CKR(pf.run(PF_RESIDUAL, s, 0, 0, 1, [&] {
            k_residual<<<P, 256, c.res_smem, s>>>(c.gv, c.pp, c.ee, all, P, w->h, nullptr, 0, nullptr, nullptr, nullptr,
                                                  w->F, w->aux, w->scal, w->r, nullptr, nullptr);
        }));
        dim3 gj(nblk(N, JAC_WARPS), P);
        cudaError_t le = cudaSuccess;
        if (prec == BTE_PREC_MIXED) {
            CKR(pf.run(PF_JACOBIAN, s, 0, 0, 1, [&] {
                const JacSmem jm = jac_smem<float>(g, c.ee);
                k_jacobian<float><<<gj, JAC_WARPS * 32, jm.bytes, s>>>(
                    c.gv, c.pp, c.ee, all, P, w->h, w->F, w->aux, w->scal, (float*)w->J, ld, js, beta, w->rowscale,
                    jm.stage, -cdt, 1.0, nullptr);
            }));
            CKR(pf.run(PF_LU, s, P * lu_flops(N), 0, 1, [&] {
                le = bte_lu_factor_t<float>(P, N, N, (float*)w->J, ld, js, w->piv, w->info, s, 0);
            }));
        } else {
            CKR(pf.run(PF_JACOBIAN, s, 0, 0, 1, [&] {
                const JacSmem jm = jac_smem<double>(g, c.ee);
                k_jacobian<double><<<gj, JAC_WARPS * 32, jm.bytes, s>>>(
                    c.gv, c.pp, c.ee, all, P, w->h, w->F, w->aux, w->scal, (double*)w->J, ld, js, beta, w->rowscale,
                    jm.stage, -cdt, 1.0, nullptr);
            }));
            CKR(pf.run(PF_LU, s, P * lu_flops(N), 0, 1, [&] {
                le = bte_lu_factor_t<double>(P, N, N, (double*)w->J, ld, js, w->piv, w->info, s, 0);
            }));
        }
        CKR(le);
        // chord iterations
        CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->refdone, 0, P); }));
        CKR(cudaMemcpyAsync(w->act, all, P * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        int nact = P;
        for (int it = 0;; ++it) {
            CKR(pf.run(PF_RESIDUAL, s, 0, 0, 1, [&] {
                k_residual<<<nact, 256, c.res_smem, s>>>(c.gv, c.pp, c.ee, w->act, nact, w->h, w->dh, ldd, w->alpha,
                                                         nullptr, w->ht, w->Ft, w->auxt, w->scalt, w->rt, nullptr,
                                                         nullptr);
            }));
            CKR(other([&] {
                k_transient_G<<<nact, 256, 0, s>>>(c.gv, nact, w->act, w->dh, ldd, w->Ft, cdt, G);
                k_ref_merit<<<nact, 256, rm_smem, s>>>(c.gv, nact, w->act, G, w->rt);
            }));
            if (it == 0) CKR(other([&] { k_copy_list<<<nblk(nact, 256), 256, 0, s>>>(nact, w->act, w->rt, w->r0); }));
            CKR(cudaMemsetAsync(w->cnt, 0, sizeof(int32_t), s));
            CKR(other([&] {
                k_transient_conv<<<nblk(nact, 256), 256, 0, s>>>(nact, w->act, w->rt, w->r0, o->atol, o->rtol,
                                                                 w->refdone, w->act2, w->cnt);
            }));
            int hn = 0;
            CKR(cudaMemcpyAsync(&hn, w->cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            CKR(cudaStreamSynchronize(s));
            pf.drain(s);
            if (hn == 0) break;
            if (it >= o->max_iter) { failed = 1; break; }
            // the points still iterating take one chord step
            if (prec == BTE_PREC_MIXED) {
                CKR(other([&] {
                    k_transient_rhs<float><<<P, 256, 0, s>>>(P, n, G, g->d_u, w->dh, ldd, beta, w->rowscale,
                                                             w->refdone, reinterpret_cast<float*>(w->xs));
                }));
                CKR(pf.run(PF_LUSOLVE, s, 0, 0, 1, [&] {
                    le = bte_lu_solve_t<float>(P, N, (const float*)w->J, ld, js, w->piv, reinterpret_cast<float*>(w->xs),
                                               0, s);
                }));
                CKR(le);
                CKR(other([&] {
                    k_transient_update<float><<<P, 256, 0, s>>>(P, n, w->refdone, reinterpret_cast<float*>(w->xs), w->dh,
                                                                ldd);
                }));
            } else {
                CKR(other([&] {
                    k_transient_rhs<double><<<P, 256, 0, s>>>(P, n, G, g->d_u, w->dh, ldd, beta, w->rowscale,
                                                              w->refdone, w->xs);
                }));
                CKR(pf.run(PF_LUSOLVE, s, 0, 0, 1, [&] {
                    le = bte_lu_solve_t<double>(P, N, (const double*)w->J, ld, js, w->piv, w->xs, 0, s);
                }));
                CKR(le);
                CKR(other([&] { k_transient_update<double><<<P, 256, 0, s>>>(P, n, w->refdone, w->xs, w->dh, ldd); }));
            }
            CKR(other([&] { k_add_iter<<<nblk(P, 256), 256, 0, s>>>(P, w->refdone, iters); }));
            std::swap(w->act, w->act2);
            nact = hn;
        }
        if (failed) break;
        if (ts > 0 && ts % io_freq == 0)
            CKR(other([&] { k_scale_into<<<nblk(P * n, 256), 256, 0, s>>>((size_t)P * n, 0.5 * o->dt, avg, avgv); }));
        CKR(other([&] { k_accumulate<<<nblk(P * n, 256), 256, 0, s>>>((size_t)P * n, w->h, avg); }));
        CKR(other([&] { k_apply_increment<<<P, 256, 0, s>>>(P, n, w->dh, ldd, w->h); }));
        CKR(other([&] { k_accumulate<<<nblk(P * n, 256), 256, 0, s>>>((size_t)P * n, w->h, avg); }));
        t += o->dt;
    }
    if (failed) CKR(other([&] { k_fill_int<<<nblk(P, 256), 256, 0, s>>>(status, BTE_ST_MAXITER, P); }));
    // outputs: the state, and the normalized distribution of the last completed cycle average
    CKR(cudaMemcpyAsync(f, w->h, (size_t)P * n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    const double c_gamma = std::sqrt(2.0 * (BTE_QE / BTE_ME));
    const double mm_fac = std::sqrt(1.0 / (4.0 * M_PI)) * 4.0 * M_PI;
    const double sc3 = 2.0 * std::pow(g->vth / c_gamma, 3);
    if (f_avg) CKR(other([&] { k_normalized_distribution<<<P, 256, 0, s>>>(n, g->d_mass, mm_fac, sc3, avgv, f_avg, P); }));
    CKR(cudaFreeAsync(all, s));
    CKR(cudaFreeAsync(Et, s));
    CKR(cudaFreeAsync(avg, s));
    CKR(cudaFreeAsync(avgv, s));
    CKR(cudaFreeAsync(G, s));
    CKR(cudaStreamSynchronize(s));
    return failed ? BTE_ERR_STATE : BTE_OK;
}
