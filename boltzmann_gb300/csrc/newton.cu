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
// merit 1/2 ||Q^T M^-1 F||^2 (:939-952) and per-point convergence.
//
//   residual   FP64 always (one CTA per point)
//   Jacobian   FP64 (plain) or FP32 (mixed) straight into the factorization buffer
//   LU         FP64 or FP32, right-hand side appended as column n+1
#include <cstdio>
#include <vector>
#include <algorithm>
#include <cmath>
#include "bte_common.cuh"
#include "bte_grid.h"

template <typename T>
cudaError_t bte_lu_factor_t(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s);
template <typename T>
cudaError_t bte_lu_solve_t(int P, int N, const T* A, int ld, long long stride, const int32_t* piv, T* b, int mode,
                           cudaStream_t s);

// device view of a grid (passed by value to kernels)
struct GridView {
    int nsp, nsh, n, lmax, nspecies, ntri;
    double vth, mw0, c_adv, gam_c, k1ev;
    const double *Mr, *Minv, *mm1, *mm2, *q0, *q1, *cgT, *adv_coef;
    const double *mass, *temp, *u, *p, *Mp, *W;
    const double *HL, *GL, *CA, *CB;
    const int* tri;
    const float *fq0, *fq1, *fcgT, *fmm1, *fmm2, *fMr, *fHL, *fGL, *fCA, *fCB;
};

struct PointParams {
    const double *n0, *ne, *Tg, *E, *ns;  // ns: n_species x P (species-major)
    int P;
};

// per-point scalar slots
enum { SC_GAMMA = 0, SC_MU, SC_T0, SC_M0, SC_NE, SC_COUNT = 8 };

// ---------------------------------------------------------------------------------
// Residual F_raw(h) for one point per CTA, plus ||(I - p p^T) M^-1 F_raw||.
// If dh != nullptr the CTA evaluates at h + alpha * dh and writes that state to hout.
// aux (if non-null) receives hh = HL h, gg = GL h, U = C_ee(h, h) raw, Mh = M h.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_residual(GridView g, PointParams pp, int ee, const int* __restrict__ act, int nact,
           const double* __restrict__ h, const double* __restrict__ dh, int ldd, const double* __restrict__ alpha,
           const int* __restrict__ need, double* hout, double* F, double* aux, double* scal, double* rnorm) {
    extern __shared__ double sm[];
    const int slot = blockIdx.x;
    if (slot >= nact) return;
    const int pt = act[slot];
    if (need && !need[pt]) return;
    const int n = g.n, nsh = g.nsh, nsp = g.nsp, tid = threadIdx.x, nt = blockDim.x;
    double* sh = sm;           // h
    double* shh = sm + n;      // HL h
    double* sgg = sm + 2 * n;  // GL h
    double* sF = sm + 3 * n;   // F_raw, later M^-1 F
    double* sR = sm + 4 * n;
    __shared__ double red[32];

    const double* hp = h + (size_t)pt * n;
    const double a = alpha ? alpha[pt] : 0.0;
    for (int i = tid; i < n; i += nt) {
        double v = hp[i];
        if (dh) v += a * dh[(size_t)pt * ldd + i];
        sh[i] = v;
        if (hout) hout[(size_t)pt * n + i] = v;
    }
    __syncthreads();
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
    for (int r = tid; r < n; r += nt) {
        const int p = r / nsh, q = r % nsh;
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
    // r = M^-1 F (block diagonal in l), projected on p-perp
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
    if (tid == 0) rnorm[pt] = sqrt(nn);
}

// ---------------------------------------------------------------------------------
// Bordered Jacobian, one warp per row, lanes along columns (row-major output):
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

template <typename T>
__global__ void __launch_bounds__(JAC_WARPS * 32)
k_jacobian(GridView g, PointParams pp, int ee, const int* __restrict__ act, int nact, const double* __restrict__ h,
           const double* __restrict__ F, const double* __restrict__ aux, const double* __restrict__ scal,
           T* __restrict__ J, int ld, long long stride, double beta_scale) {
    const int slot = blockIdx.y;
    if (slot >= nact) return;
    const int pt = act[slot];
    const int n = g.n, nsh = g.nsh, nsp = g.nsp, N = n + 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int a = blockIdx.x * JAC_WARPS + wid;  // row
    if (a > n) return;
    T* Jr = J + (size_t)slot * stride + (size_t)a * ld;
    const double* hp = h + (size_t)pt * n;
    const double* ax = aux + (size_t)pt * 4 * n;
    const double* sc = scal + (size_t)pt * SC_COUNT;
    const double n0 = pp.n0[pt], Tg = pp.Tg[pt], E = pp.E[pt];
    const double beta = beta_scale * n0;
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
    // K2a[dr][s], K2b[dr][s] for this row: sum over triples (q, l, s) and dk of C[t][p][dk][dr] h[(p+dk, l)]
    const T* CA = OpsT<T>::CA(g);
    const T* CB = OpsT<T>::CB(g);
    T k2a[BTE_NB * 5], k2b[BTE_NB * 5];  // l_max <= 4
    if (ee) {
#pragma unroll
        for (int i = 0; i < BTE_NB * 5; ++i) { k2a[i] = T(0); k2b[i] = T(0); }
        for (int t = 0; t < g.ntri; ++t) {
            if (g.tri[3 * t] != q) continue;
            const int l = g.tri[3 * t + 1], s = g.tri[3 * t + 2];
            const T* ca = CA + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
            const T* cb = CB + ((size_t)t * nsp + p) * BTE_NB * BTE_NB;
            for (int dk = -BTE_BAND; dk <= BTE_BAND; ++dk) {
                int k = p + dk;
                if (k < 0 || k >= nsp) continue;
                T hv = (T)hp[k * nsh + l];
#pragma unroll
                for (int dr = 0; dr < BTE_NB; ++dr) {
                    int o = (dk + BTE_BAND) * BTE_NB + dr;
                    // s is bounded by l_max <= 4, index computed at run time
                    k2a[s * BTE_NB + dr] += ca[o] * hv;
                    k2b[s * BTE_NB + dr] += cb[o] * hv;
                }
            }
        }
    }
    const T* HL = OpsT<T>::HL(g);
    const T* GL = OpsT<T>::GL(g);
    const T* q0 = OpsT<T>::q0(g);
    const T* q1 = OpsT<T>::q1(g);
    const T* cgT = OpsT<T>::cgT(g);
    const T* mm1 = OpsT<T>::mm1(g);
    const T* mm2 = OpsT<T>::mm2(g);
    const T* Mr = OpsT<T>::Mr(g);
    const double cadv = E * g.c_adv;
    for (int j = lane; j < N + 1; j += 32) {
        if (j == n) { Jr[j] = (T)(-beta * g.Mp[a]); continue; }
        if (j == n + 1) { Jr[j] = (T)(-F[(size_t)pt * n + a]); continue; }
        const int c = j / nsh, s = j % nsh;
        T v = T(0);
        double wj = 0.0;
        if (s == 0)
            for (int sp = 0; sp < g.nspecies; ++sp) wj += n0 * pp.ns[(size_t)sp * pp.P + pt] * g.W[(size_t)sp * n + j];
        double dgj = ee ? (dg_t * g.temp[j] * g.k1ev - dg_m * g.mass[j]) : 0.0;
        v += (T)(-mh * wj + dgj);
        if (ee) {
            const T* hl = HL + (size_t)s * nsp * nsp + c;
            const T* gl = GL + (size_t)s * nsp * nsp + c;
            T acc = T(0);
#pragma unroll
            for (int dr = 0; dr < BTE_NB; ++dr) {
                int r = p + dr - BTE_BAND;
                if (r < 0 || r >= nsp) continue;
                acc += k2a[s * BTE_NB + dr] * hl[(size_t)r * nsp] + k2b[s * BTE_NB + dr] * gl[(size_t)r * nsp];
            }
            v += (T)negam * acc;
        }
        // l = 0 collision block (not banded: v_post shifts the support)
        if (q == 0 && s == 0)
            for (int sp = 0; sp < g.nspecies; ++sp)
                v += (T)(n0 * pp.ns[(size_t)sp * pp.P + pt]) * q0[((size_t)sp * nsp + p) * nsp + c];
        const int dk = c - p;
        if (dk >= -BTE_BAND && dk <= BTE_BAND) {
            const int bi = p * BTE_NB + dk + BTE_BAND;
            if (s == q) {
                if (q == 0) v += (T)(n0 * Tg) * cgT[bi];
                else
                    for (int sp = 0; sp < g.nspecies; ++sp)
                        v += (T)(n0 * pp.ns[(size_t)sp * pp.P + pt]) * q1[((size_t)sp * nsp + p) * BTE_NB + dk + BTE_BAND];
                v -= (T)mu * Mr[bi];
            }
            if (s == q + 1)
                v += (T)cadv * (mm1[bi] * (T)g.adv_coef[q * 4 + 0] + (T)g.adv_coef[q * 4 + 1] * mm2[bi]);
            if (s == q - 1)
                v += (T)cadv * (mm1[bi] * (T)g.adv_coef[q * 4 + 2] + (T)g.adv_coef[q * 4 + 3] * mm2[bi]);
            if (ee) {
                // K1[(p,q)][(c,s)] = sum_{t=(q,s,s')} sum_dr C[t][p][dk][dr] pot[(p+dr, s')]
                T k1 = T(0);
                for (int t = 0; t < g.ntri; ++t) {
                    if (g.tri[3 * t] != q || g.tri[3 * t + 1] != s) continue;
                    const int s2 = g.tri[3 * t + 2];
                    const T* ca = CA + ((size_t)t * nsp + p) * BTE_NB * BTE_NB + (dk + BTE_BAND) * BTE_NB;
                    const T* cb = CB + ((size_t)t * nsp + p) * BTE_NB * BTE_NB + (dk + BTE_BAND) * BTE_NB;
                    for (int dr = -BTE_BAND; dr <= BTE_BAND; ++dr) {
                        int rr = p + dr;
                        if (rr < 0 || rr >= nsp) continue;
                        k1 += ca[dr + BTE_BAND] * (T)ax[rr * nsh + s2] + cb[dr + BTE_BAND] * (T)ax[n + rr * nsh + s2];
                    }
                }
                v += (T)negam * k1;
            }
        }
        Jr[j] = v;
    }
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

// Armijo test (bte_0d3v_batched.py:942-952) for every point still searching
__global__ void k_armijo(int nact, const int* __restrict__ act, int* searching, double* alpha,
                         const double* __restrict__ r, const double* __restrict__ rt, double c, double rho,
                         double amin, int* status, int* nsearch, int* accepted, const double* __restrict__ r0,
                         double stagnate_rtol) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    if (!searching[pt]) return;
    double rr = r[pt], rn = rt[pt], al = alpha[pt];
    bool ok = (0.5 * rn * rn <= 0.5 * rr * rr - c * al * rr * rr);
    if (!isfinite(rn)) ok = false;
    if (ok) {
        searching[pt] = 0;
        accepted[pt] = 1;
        return;
    }
    // at round-off level a full step that does not decrease the merit ends the solve
    if (al == 1.0 && rr <= stagnate_rtol * r0[pt]) {
        searching[pt] = 0;
        accepted[pt] = 0;
        status[pt] = BTE_ST_ROUNDOFF;
        return;
    }
    al *= rho;
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
__global__ void k_converge(int nact, const int* __restrict__ act, const double* __restrict__ r,
                           const double* __restrict__ r0, double atol, double rtol, int last, int* status,
                           int* act_out, int* nout, const int32_t* __restrict__ info, int check_info) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nact) return;
    int pt = act[slot];
    int st = status[pt];
    if (st < 0) {
        if (!isfinite(r[pt])) st = BTE_ST_NONFINITE;
        else if (r[pt] <= atol + rtol * r0[pt]) st = BTE_ST_CONVERGED;
        else if (check_info && info[slot] != 0) st = BTE_ST_SINGULAR;
        else if (last) st = BTE_ST_MAXITER;
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
    void* J = nullptr;
    int32_t *piv = nullptr, *info = nullptr, *act = nullptr, *act2 = nullptr, *cnt = nullptr;
    int32_t *searching = nullptr, *accepted = nullptr;
};

static void free_work(BteWork* w) {
    void* ptrs[] = {w->xs, w->h, w->ht, w->F, w->Ft, w->aux, w->auxt, w->scal, w->scalt, w->dh, w->r, w->rt, w->r0,
                    w->alpha, w->J, w->piv, w->info, w->act, w->act2, w->cnt, w->searching, w->accepted};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    *w = BteWork();
}

static GridView view_of(const BteGrid* g) {
    GridView v;
    v.nsp = g->nsp; v.nsh = g->nsh; v.n = g->n; v.lmax = g->lmax; v.nspecies = g->nspecies; v.ntri = g->ntri;
    v.vth = g->vth; v.mw0 = g->mw0; v.c_adv = g->c_adv;
    v.gam_c = (BTE_QE * BTE_QE * BTE_QE * BTE_QE) / (4.0 * BTE_PI * (BTE_EPS0 * BTE_ME) * (BTE_EPS0 * BTE_ME)) / (g->vth * g->vth * g->vth);
    v.k1ev = BTE_QE / BTE_KB;
    v.Mr = g->d_Mr; v.Minv = g->d_Minv; v.mm1 = g->d_mm1; v.mm2 = g->d_mm2; v.q0 = g->d_q0; v.q1 = g->d_q1;
    v.cgT = g->d_cgT; v.adv_coef = g->d_adv_coef; v.mass = g->d_mass; v.temp = g->d_temp; v.u = g->d_u; v.p = g->d_p;
    v.Mp = g->d_Mp; v.W = g->d_W; v.HL = g->d_HL; v.GL = g->d_GL; v.CA = g->d_CA; v.CB = g->d_CB; v.tri = g->d_tri;
    v.fq0 = g->f_q0; v.fq1 = g->f_q1; v.fcgT = g->f_cgT; v.fmm1 = g->f_mm1; v.fmm2 = g->f_mm2; v.fMr = g->f_Mr;
    v.fHL = g->f_HL; v.fGL = g->f_GL; v.fCA = g->f_CA; v.fCB = g->f_CB;
    return v;
}

#define CKR(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { fprintf(stderr, "bte: %s at %s:%d\n", cudaGetErrorString(_e), __FILE__, __LINE__); return BTE_ERR_CUDA; } } while (0)

static int ensure_work(BteWork* w, const BteGrid* g, int P, int prec) {
    const int n = g->n, N = n + 1;
    const int ld = (N + 1 + 3) & ~3;  // row length of the augmented matrix, padded
    size_t jb = (size_t)P * N * ld * (prec == BTE_PREC_MIXED ? sizeof(float) : sizeof(double));
    if (w->cap >= P && w->n == n && w->jbytes >= jb) return BTE_OK;
    free_work(w);
    auto A = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, std::max<size_t>(bytes, 8)) == cudaSuccess; };
    size_t pn = (size_t)P * n * sizeof(double);
    bool ok = A((void**)&w->h, pn) && A((void**)&w->ht, pn) && A((void**)&w->F, pn) && A((void**)&w->Ft, pn) &&
              A((void**)&w->aux, 4 * pn) && A((void**)&w->auxt, 4 * pn) &&
              A((void**)&w->scal, (size_t)P * SC_COUNT * sizeof(double)) &&
              A((void**)&w->scalt, (size_t)P * SC_COUNT * sizeof(double)) &&
              A((void**)&w->dh, (size_t)P * (N + 1) * sizeof(double)) &&
              A((void**)&w->xs, (size_t)P * (N + 1) * sizeof(double)) && A((void**)&w->r, P * sizeof(double)) &&
              A((void**)&w->rt, P * sizeof(double)) && A((void**)&w->r0, P * sizeof(double)) &&
              A((void**)&w->alpha, P * sizeof(double)) && A(&w->J, jb) &&
              A((void**)&w->piv, (size_t)P * N * sizeof(int32_t)) && A((void**)&w->info, P * sizeof(int32_t)) &&
              A((void**)&w->act, P * sizeof(int32_t)) && A((void**)&w->act2, P * sizeof(int32_t)) &&
              A((void**)&w->cnt, 4 * sizeof(int32_t)) && A((void**)&w->searching, P * sizeof(int32_t)) &&
              A((void**)&w->accepted, P * sizeof(int32_t));
    if (!ok) { free_work(w); return BTE_ERR_ALLOC; }
    w->cap = P; w->n = n; w->jbytes = jb; w->prec = prec;
    return BTE_OK;
}

static inline unsigned nblk(int n, int b) { return (unsigned)((n + b - 1) / b); }

BteWork* bte_work_get(BteGrid* g) {
    if (!g->work) g->work = new BteWork();
    return g->work;
}
void bte_work_release(BteWork* w) {
    if (w) { free_work(w); delete w; }
}

int bte_solve_impl(BteGrid* g, int P, const double* n0, const double* ne, const double* ns_by_n0, const double* Tg,
                   const double* E, double* f, int32_t* status, int32_t* iters, const bte_solve_opts* o,
                   cudaStream_t s) {
    if (P <= 0) return BTE_OK;
    BteWork* w = bte_work_get(g);
    const int prec = o->precision;
    int rc = ensure_work(w, g, P, prec);
    if (rc) return rc;
    const int n = g->n, N = n + 1;
    const int ld = (N + 1 + 3) & ~3;
    const long long jstride = (long long)N * ld;
    const int ee = (o->ee && g->ee) ? 1 : 0;
    GridView gv = view_of(g);
    PointParams pp{n0, ne, Tg, E, ns_by_n0, P};
    // border scale: typical magnitude of the raw collision operator per unit n0
    const double beta_scale = g->q0max / (g->umax > 0 ? g->umax : 1.0);
    const size_t res_smem = (size_t)5 * n * sizeof(double);
    if (res_smem > 48 * 1024) CKR(cudaFuncSetAttribute(k_residual, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)res_smem));

    k_mass_normalize<<<P, 256, 0, s>>>(n, g->d_u, f, w->h, P);
    k_fill_int<<<nblk(P, 256), 256, 0, s>>>(status, -1, P);
    k_fill_int<<<nblk(P, 256), 256, 0, s>>>(iters, 0, P);
    k_iota<<<nblk(P, 256), 256, 0, s>>>(w->act, P);
    CKR(cudaGetLastError());
    k_residual<<<P, 256, res_smem, s>>>(gv, pp, ee, w->act, P, w->h, nullptr, 0, nullptr, nullptr, nullptr, w->F,
                                        w->aux, w->scal, w->r);
    CKR(cudaGetLastError());
    CKR(cudaMemcpyAsync(w->r0, w->r, P * sizeof(double), cudaMemcpyDeviceToDevice, s));
    int nact = P;
    const int ldd = N + 1;
    for (int it = 0; it < o->max_iter && nact > 0; ++it) {
        // Jacobian straight into the factorization buffer, then LU of [J | -F]
        dim3 gj(nblk(N, JAC_WARPS), nact);
        if (prec == BTE_PREC_MIXED) {
            k_jacobian<float><<<gj, JAC_WARPS * 32, 0, s>>>(gv, pp, ee, w->act, nact, w->h, w->F, w->aux, w->scal,
                                                              (float*)w->J, ld, jstride, beta_scale);
            CKR(cudaGetLastError());
            CKR(bte_lu_factor_t<float>(nact, N, N + 1, (float*)w->J, ld, jstride, w->piv, w->info, s));
        } else {
            k_jacobian<double><<<gj, JAC_WARPS * 32, 0, s>>>(gv, pp, ee, w->act, nact, w->h, w->F, w->aux, w->scal,
                                                               (double*)w->J, ld, jstride, beta_scale);
            CKR(cudaGetLastError());
            CKR(bte_lu_factor_t<double>(nact, N, N + 1, (double*)w->J, ld, jstride, w->piv, w->info, s));
        }
        // back substitution into dh (FP64 buffer indexed by point)
        if (prec == BTE_PREC_MIXED) {
            float* xs = reinterpret_cast<float*>(w->xs);
            CKR(bte_lu_solve_t<float>(nact, N, (const float*)w->J, ld, jstride, w->piv, xs, 1, s));
            k_store_solution<float><<<nact, 128, 0, s>>>(nact, xs, N, w->act, w->dh, ldd);
        } else {
            double* xs = w->xs;
            CKR(bte_lu_solve_t<double>(nact, N, (const double*)w->J, ld, jstride, w->piv, xs, 1, s));
            k_store_solution<double><<<nact, 128, 0, s>>>(nact, xs, N, w->act, w->dh, ldd);
        }
        CKR(cudaGetLastError());
        // line search
        k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->searching, 0, P);
        k_fill_int<<<nblk(P, 256), 256, 0, s>>>(w->accepted, 0, P);
        k_set_active<<<nblk(nact, 256), 256, 0, s>>>(nact, w->act, w->searching, w->alpha);
        for (int ls = 0; ls < 200; ++ls) {
            k_residual<<<nact, 256, res_smem, s>>>(gv, pp, ee, w->act, nact, w->h, w->dh, ldd, w->alpha, w->searching,
                                                   w->ht, w->Ft, w->auxt, w->scalt, w->rt);
            CKR(cudaMemsetAsync(w->cnt, 0, sizeof(int32_t), s));
            k_armijo<<<nblk(nact, 256), 256, 0, s>>>(nact, w->act, w->searching, w->alpha, w->r, w->rt, o->line_search_c,
                                                    o->alpha_rho, o->alpha_min, status, w->cnt, w->accepted, w->r0, 1e-9);
            CKR(cudaGetLastError());
            int hc = 0;
            CKR(cudaMemcpyAsync(&hc, w->cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            CKR(cudaStreamSynchronize(s));
            if (hc == 0) break;
        }
        k_accept<<<nact, 256, 0, s>>>(n, nact, w->act, w->accepted, w->h, w->ht, w->F, w->Ft, w->aux, w->auxt, w->scal,
                                     w->scalt, w->r, w->rt, iters);
        CKR(cudaMemsetAsync(w->cnt, 0, sizeof(int32_t), s));
        k_converge<<<nblk(nact, 256), 256, 0, s>>>(nact, w->act, w->r, w->r0, o->atol, o->rtol,
                                                  it + 1 == o->max_iter, status, w->act2, w->cnt, w->info, 0);
        CKR(cudaGetLastError());
        int hn = 0;
        CKR(cudaMemcpyAsync(&hn, w->cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        CKR(cudaStreamSynchronize(s));
        std::swap(w->act, w->act2);
        nact = hn;
    }
    const double c_gamma = std::sqrt(2.0 * (BTE_QE / BTE_ME));
    const double mm_fac = std::sqrt(1.0 / (4.0 * M_PI)) * 4.0 * M_PI;
    const double sc3 = 2.0 * std::pow(g->vth / c_gamma, 3);
    k_normalized_distribution<<<P, 256, 0, s>>>(n, g->d_mass, mm_fac, sc3, w->h, f, P);
    CKR(cudaGetLastError());
    return BTE_OK;
}
