// 1D3V spatially coupled step of the velocity-space solver (sm_103a): the spectral
// (B-spline x spherical harmonic) v-space with discrete ordinates in v-theta and Chebyshev
// collocation in x, advanced by the reference's Strang split
// (bte_1d3v_solver.py:1885-1889): x-advection half step, v-space step, x-advection half step.
//
// State layouts on the device (double):
//   ordinates  V[(r * Nvt + j) * Nx + x]      r radial coefficient, j ordinate, x Chebyshev point
//                                             (the reference's (Nr * Nvt, Nx) array)
//   v-space    U[x * n + (r * nsh + l)]       x-major: each point's n = Nr * nsh coefficients
//                                             contiguous, so per-point blocks are contiguous
//
// x-step (step_bte_x, bte_1d3v_solver.py:912-982, BE Chebyshev form): V' = Q^-1 V in the radial
// index (adv_x = Q diag(d) Q^-1), inflow values zeroed (x = -1 for cos(theta) >= 0, x = +1
// otherwise), one backward-Euler solve (I + h d_r cos(theta_j) D_L/R) per (r, j) over x, and
// V = Q V'. The Nr * Nvt matrices are inverted once per step size (LU factors, then one
// identity column per pass), so each step is an HBM-bound batched product with the inverses.
//
// v-step (step_bte_v, bte_1d3v_solver.py:984-1137): U = P_o2sh V, then
//   (I - dt (Cv + E_x Av)) U_new = U  at every x (Cv = tau n0 np0 (C_en + Tg C_gT), Av = tau A,
//   all M^-1-scaled), solved by right-preconditioned restarted GMRES (utils.py:1172-1262) whose
//   matvec is the fused Lmat_mvec (bte_1d3v_solver.py:1051-1055) and whose preconditioner is the
//   block inverse of each x point's own matrix, factored in FP32 (the reference uses the
//   inverse of the nearest of num_pc_ops E values instead, :889-910,1057-1064); V = P_sh2o U.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>
#include <string>
#include <algorithm>
#include "bte_common.cuh"
#include "bte_grid.h"
#include "../../include/bte1d_gb300.h"

template <typename T>
cudaError_t bte_lu_factor_t(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s, int kernel);
template <typename T>
cudaError_t bte_lu_solve_t(int P, int N, const T* A, int ld, long long stride, const int32_t* piv, T* b, int mode,
                           cudaStream_t s, const int32_t* mats = nullptr);

namespace {

constexpr int RED_BLOCKS = 120;   // partial-sum blocks of the reductions (deterministic order)

// out[i][c] = sum_k Qm[i][k] in[k][c], i, k < Nr, c < C (C = Nvt * Nx): the radial basis change
__global__ void k_radial_mix(int Nr, int C, const double* __restrict__ Qm, const double* __restrict__ in,
                             double* __restrict__ out) {
    extern __shared__ double sq[];
    for (int e = threadIdx.x; e < Nr * Nr; e += blockDim.x) sq[e] = Qm[e];
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (c >= C) return;
    double s = 0.0;
    for (int k = 0; k < Nr; ++k) s += sq[i * Nr + k] * in[(size_t)k * C + c];
    out[(size_t)i * C + c] = s;
}

// inflow boundary values: x = 0 (x = -1) for ordinates moving right, x = Nx - 1 for the others
__global__ void k_zero_inflow(int Nr, int Nvt, int Nx, const int8_t* __restrict__ right, double* V) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Nr * Nvt) return;
    const int j = e % Nvt;
    V[(size_t)e * Nx + (right[j] ? 0 : Nx - 1)] = 0.0;
}

// A[(r * Nvt + j)] = I + h d_r cos(theta_j) D_X, D_L = D with row 0 zeroed (right-moving
// ordinates), D_R = D with row Nx - 1 zeroed
__global__ void k_build_xshift(int Nr, int Nvt, int Nx, double h, const double* __restrict__ d,
                               const double* __restrict__ cth, const int8_t* __restrict__ right,
                               const double* __restrict__ D, double* A, int ld, long long stride) {
    const int m = blockIdx.y;
    const int r = m / Nvt, j = m % Nvt;
    const double f = h * d[r] * cth[j];
    const int zrow = right[j] ? 0 : Nx - 1;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Nx * Nx; e += gridDim.x * blockDim.x) {
        const int a = e / Nx, b = e % Nx;
        double v = (a == zrow) ? 0.0 : f * D[(size_t)a * Nx + b];
        if (a == b) v += 1.0;
        A[(size_t)m * stride + (size_t)a * ld + b] = v;
    }
}

// right-hand sides e_c for every system (column c of the identity)
__global__ void k_unit_rhs(int P, int Nx, int c, double* B) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)P * Nx) return;
    B[e] = ((int)(e % Nx) == c) ? 1.0 : 0.0;
}
// column c of each inverse, stored as row c of its transpose: XT[m][c][:] = x_m
__global__ void k_store_invcol(int P, int Nx, int c, const double* __restrict__ B, double* XT) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)P * Nx) return;
    const size_t m = e / Nx, i = e % Nx;
    XT[(m * Nx + c) * Nx + i] = B[e];
}
// out[m][i] = sum_k A^-1[m][i][k] in[m][k] with the transposed inverse XT[m][k][i]: one CTA
// per system, threads along i (coalesced rows of XT), in[m][:] staged in shared memory
__global__ void __launch_bounds__(256) k_xstep_apply(int Nx, const double* __restrict__ XT,
                                                     const double* __restrict__ in, double* __restrict__ out) {
    extern __shared__ double sv[];
    const int m = blockIdx.x;
    const double* A = XT + (size_t)m * Nx * Nx;
    for (int k = threadIdx.x; k < Nx; k += blockDim.x) sv[k] = in[(size_t)m * Nx + k];
    __syncthreads();
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) {
        double acc = 0.0;
#pragma unroll 4
        for (int k = 0; k < Nx; ++k) acc += A[(size_t)k * Nx + i] * sv[k];
        out[(size_t)m * Nx + i] = acc;
    }
}

// ordinates -> spherical harmonics, into the x-major layout: U[x][r nsh + l] = sum_j Ps[l][j] V[r][j][x]
__global__ void k_ords_to_lm(int Nr, int Nvt, int nsh, int Nx, const double* __restrict__ Ps,
                             const double* __restrict__ V, double* __restrict__ U) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Nr * nsh * Nx) return;
    const int x = e % Nx, a = e / Nx, r = a / nsh, l = a % nsh;
    double s = 0.0;
    for (int j = 0; j < Nvt; ++j) s += Ps[l * Nvt + j] * V[((size_t)r * Nvt + j) * Nx + x];
    U[(size_t)x * (Nr * nsh) + a] = s;
}

// spherical harmonics -> ordinates: V[r][j][x] = sum_l Po[j][l] U[x][r nsh + l]
__global__ void k_lm_to_ords(int Nr, int Nvt, int nsh, int Nx, const double* __restrict__ Po,
                             const double* __restrict__ U, double* __restrict__ V) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Nr * Nvt * Nx) return;
    const int x = e % Nx, rj = e / Nx, r = rj / Nvt, j = rj % Nvt;
    double s = 0.0;
    for (int l = 0; l < nsh; ++l) s += Po[j * nsh + l] * U[(size_t)x * (Nr * nsh) + r * nsh + l];
    V[e] = s;
}

// Lmat_mvec (bte_1d3v_solver.py:1051-1055) in the x-major layout:
//   Y[x][a] = X[x][a] - dt (sum_b Cv[a][b] X[x][b] + E[x] sum_b Av[a][b] X[x][b])
// CvT / AvT are stored transposed so that the threads of a CTA (one per a) read along a.
constexpr int MV_X = 8;
__global__ void __launch_bounds__(256)
k_lmat(int n, int Nx, double dt, const double* __restrict__ CvT, const double* __restrict__ AvT,
       const double* __restrict__ E, const double* __restrict__ X, double* __restrict__ Y) {
    extern __shared__ double sx[];  // [MV_X][n]
    const int x0 = blockIdx.x * MV_X;
    const int nx = min(MV_X, Nx - x0);
    for (int e = threadIdx.x; e < nx * n; e += blockDim.x) sx[e] = X[(size_t)x0 * n + e];
    __syncthreads();
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        double c[MV_X], v[MV_X];
#pragma unroll
        for (int t = 0; t < MV_X; ++t) { c[t] = 0.0; v[t] = 0.0; }
        for (int b = 0; b < n; ++b) {
            const double cb = CvT[(size_t)b * n + a], ab = AvT[(size_t)b * n + a];
#pragma unroll
            for (int t = 0; t < MV_X; ++t) {
                const double xb = (t < nx) ? sx[t * n + b] : 0.0;
                c[t] += cb * xb;
                v[t] += ab * xb;
            }
        }
#pragma unroll
        for (int t = 0; t < MV_X; ++t)
            if (t < nx) Y[(size_t)(x0 + t) * n + a] = sx[t * n + a] - dt * (c[t] + E[x0 + t] * v[t]);
    }
}

// the per-point blocks I - dt (Cv + E_x Av), FP32, row-major with leading dimension ld
__global__ void k_build_vblocks(int n, int Nx, double dt, const double* __restrict__ CvT,
                                const double* __restrict__ AvT, const double* __restrict__ E, float* B, int ld,
                                long long stride) {
    const int x = blockIdx.y;
    const double Ex = E[x];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
        const int a = e / n, b = e % n;
        double v = -dt * (CvT[(size_t)b * n + a] + Ex * AvT[(size_t)b * n + a]);
        if (a == b) v += 1.0;
        B[(size_t)x * stride + (size_t)a * ld + b] = (float)v;
    }
}

__global__ void k_to_f32(size_t m, const double* __restrict__ a, float* __restrict__ b) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) b[i] = (float)a[i];
}
__global__ void k_to_f64(size_t m, const float* __restrict__ a, double* __restrict__ b) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) b[i] = (double)a[i];
}

// partial dot products of k vectors (stride ld) with w: part[j][block]
__global__ void k_dots_partial(size_t m, int k, const double* __restrict__ V, size_t ldv,
                               const double* __restrict__ w, double* part) {
    __shared__ double red[32];
    const int j = blockIdx.y;
    const double* v = V + (size_t)j * ldv;
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
        s += v[i] * w[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = s;
}
__global__ void k_dots_final(int k, int nb, const double* __restrict__ part, double* out) {
    __shared__ double red[32];
    const int j = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[(size_t)j * nb + i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) out[j] = s;
}

// w -= sum_j h[j] V_j  (h on the device)
__global__ void k_sub_combo(size_t m, int k, const double* __restrict__ V, size_t ldv, const double* __restrict__ h,
                            double* w) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double s = w[i];
    for (int j = 0; j < k; ++j) s -= h[j] * V[(size_t)j * ldv + i];
    w[i] = s;
}
// y = sum_j c[j] V_j
__global__ void k_combo(size_t m, int k, const double* __restrict__ V, size_t ldv, const double* __restrict__ c,
                        double* y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += c[j] * V[(size_t)j * ldv + i];
    y[i] = s;
}
__global__ void k_scale(size_t m, double a, const double* __restrict__ x, double* y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) y[i] = a * x[i];
}
__global__ void k_axpy(size_t m, double a, const double* __restrict__ x, double* y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) y[i] += a * x[i];
}
__global__ void k_sub(size_t m, const double* __restrict__ a, const double* __restrict__ b, double* c) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) c[i] = a[i] - b[i];
}

inline unsigned nb(size_t m, int b) { return (unsigned)((m + b - 1) / b); }

// ---- fully implicit spectral step ------------------------------------------------------------
// T[m][x] = sum_k D[x][k] V[m][k] for each (r, j) line m = r * Nvt + j, with the inflow row of
// the upwinded derivative zeroed (row 0 for ordinates moving right, D_L; row Nx - 1 otherwise,
// D_R: bte_1d3v_solver.py:792-800). DT = D transposed, so that the threads (one per output x)
// read consecutive entries; each entry feeds FD_L lines staged in shared memory.
constexpr int FD_L = 8;
__global__ void __launch_bounds__(256)
k_fim_dx(int Nlines, int Nvt, int Nx, const double* __restrict__ DT, const int8_t* __restrict__ right,
         const double* __restrict__ V, double* __restrict__ T) {
    extern __shared__ double sv[];  // [FD_L][Nx]
    const int l0 = blockIdx.x * FD_L;
    const int nl = min(FD_L, Nlines - l0);
    for (int e = threadIdx.x; e < nl * Nx; e += blockDim.x) sv[e] = V[(size_t)l0 * Nx + e];
    __syncthreads();
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        double acc[FD_L];
#pragma unroll
        for (int t = 0; t < FD_L; ++t) acc[t] = 0.0;
        for (int k = 0; k < Nx; ++k) {
            const double dk = DT[(size_t)k * Nx + x];
#pragma unroll
            for (int t = 0; t < FD_L; ++t) acc[t] += dk * sv[(t < nl ? t : 0) * Nx + k];
        }
#pragma unroll
        for (int t = 0; t < FD_L; ++t) {
            if (t >= nl) break;
            const int j = (l0 + t) % Nvt;
            const bool inflow_row = right[j] ? (x == 0) : (x == Nx - 1);
            T[(size_t)(l0 + t) * Nx + x] = inflow_row ? 0.0 : acc[t];
        }
    }
}

// The backward-Euler operator of the fully implicit step on ordinates, per x point:
//   Y = V - dt (P_sh2o (Cv + E_x Av) P_o2sh V - cos(theta_j) adv_x T)
// (T = the x-derivative lines of k_fim_dx; Cv, Av carry tau), with identity rows on the inflow
// boundary. One CTA per FC_X consecutive x points; V, T, adv_x staged in shared memory.
constexpr int FC_X = 1;   // one x point per CTA: Nx CTAs (the radial mixing dominates)
__global__ void __launch_bounds__(256)
k_fim_combine(int Nr, int Nvt, int nsh, int Nx, double dt, const double* __restrict__ Ps,
              const double* __restrict__ Po, const double* __restrict__ CvT, const double* __restrict__ AvT,
              const double* __restrict__ AxT, const double* __restrict__ cth, const int8_t* __restrict__ right,
              const double* __restrict__ E, const double* __restrict__ V, const double* __restrict__ T,
              double* __restrict__ Y) {
    extern __shared__ double sm[];
    const int M = Nr * Nvt, n = Nr * nsh;
    double* sV = sm;                 // [FC_X][M]
    double* sT = sV + FC_X * M;      // [FC_X][M]
    double* sU = sT + FC_X * M;      // [FC_X][n]  harmonics
    double* sW = sU + FC_X * n;      // [FC_X][n]  (Cv + E Av) harmonics
    double* sA = sW + FC_X * n;      // [Nr][Nr]   adv_x transposed
    const int x0 = blockIdx.x * FC_X;
    const int nx = min(FC_X, Nx - x0);
    for (int e = threadIdx.x; e < M * FC_X; e += blockDim.x) {
        const int m = e / FC_X, t = e % FC_X;
        const bool ok = t < nx;
        sV[t * M + m] = ok ? V[(size_t)m * Nx + x0 + t] : 0.0;
        sT[t * M + m] = ok ? T[(size_t)m * Nx + x0 + t] : 0.0;
    }
    for (int e = threadIdx.x; e < Nr * Nr; e += blockDim.x) sA[e] = AxT[e];
    __syncthreads();
    for (int e = threadIdx.x; e < n * FC_X; e += blockDim.x) {
        const int a = e % n, t = e / n, r = a / nsh, l = a % nsh;
        double u = 0.0;
        for (int j = 0; j < Nvt; ++j) u += Ps[l * Nvt + j] * sV[t * M + r * Nvt + j];
        sU[t * n + a] = u;
    }
    __syncthreads();
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        double c[FC_X], v[FC_X];
#pragma unroll
        for (int t = 0; t < FC_X; ++t) { c[t] = 0.0; v[t] = 0.0; }
        for (int b = 0; b < n; ++b) {
            const double cb = CvT[(size_t)b * n + a], ab = AvT[(size_t)b * n + a];
#pragma unroll
            for (int t = 0; t < FC_X; ++t) {
                c[t] += cb * sU[t * n + b];
                v[t] += ab * sU[t * n + b];
            }
        }
#pragma unroll
        for (int t = 0; t < FC_X; ++t) sW[t * n + a] = c[t] + ((t < nx) ? E[x0 + t] : 0.0) * v[t];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < M * FC_X; e += blockDim.x) {
        const int t = e / M, m = e % M, r = m / Nvt, j = m % Nvt;
        if (t >= nx) continue;
        const int x = x0 + t;
        const double vx = sV[t * M + m];
        const bool inflow_row = right[j] ? (x == 0) : (x == Nx - 1);
        double y = vx;
        if (!inflow_row) {
            double yv = 0.0;
            for (int l = 0; l < nsh; ++l) yv += Po[j * nsh + l] * sW[t * n + r * nsh + l];
            double yx = 0.0;
            for (int k = 0; k < Nr; ++k) yx += sA[k * Nr + r] * sT[t * M + k * Nvt + j];
            y = vx - dt * (yv - cth[j] * yx);
        }
        Y[(size_t)m * Nx + x] = y;
    }
}

// out = in + P_sh2o (Z - U): the exact inverse of I - dt P_sh2o L_v P_o2sh on ordinates from the
// per-point inverse Z = (I - dt L_v)^-1 U of the harmonics U = P_o2sh in (P_o2sh P_sh2o = I)
__global__ void k_lm_correct(int Nr, int Nvt, int nsh, int Nx, const double* __restrict__ Po,
                             const double* __restrict__ in, const double* __restrict__ Z,
                             const double* __restrict__ U, double* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Nr * Nvt * Nx) return;
    const int x = e % Nx, rj = e / Nx, r = rj / Nvt, j = rj % Nvt;
    double s = in[e];
    for (int l = 0; l < nsh; ++l) {
        const size_t a = (size_t)x * (Nr * nsh) + r * nsh + l;
        s += Po[j * nsh + l] * (Z[a] - U[a]);
    }
    out[e] = s;
}

// copy with the inflow boundary values set to 0
__global__ void k_copy_zero_inflow(int Nr, int Nvt, int Nx, const int8_t* __restrict__ right,
                                   const double* __restrict__ in, double* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Nr * Nvt * Nx) return;
    const int x = e % Nx, j = (e / Nx) % Nvt;
    const bool inflow = right[j] ? (x == 0) : (x == Nx - 1);
    out[e] = inflow ? 0.0 : in[e];
}

}  // namespace

struct Bte1d {
    int device = 0;
    int Nr = 0, nsh = 0, n = 0, Nvt = 0, Nx = 0;
    // setup operators (device)
    double *Q = nullptr, *Qinv = nullptr, *d = nullptr, *cth = nullptr, *D = nullptr;
    double *Ps = nullptr, *Po = nullptr, *CvT = nullptr, *AvT = nullptr;
    int8_t* right = nullptr;
    // x-step factors
    double hx = -1.0;
    double* XA = nullptr;
    double* XI = nullptr;  // transposed inverses of the x-step matrices, Nr * Nvt x Nx x Nx
    int32_t *Xpiv = nullptr, *Xinfo = nullptr;
    int xld = 0;
    // v-step buffers
    float* VB = nullptr;
    int32_t *Vpiv = nullptr, *Vinfo = nullptr;
    int vld = 0;
    double *U = nullptr, *R = nullptr, *W = nullptr, *Z = nullptr, *Xs = nullptr, *T = nullptr;
    float* Zf = nullptr;
    double* Kr = nullptr;  // Krylov basis, (restart + 1) vectors
    int kcap = 0;
    double *part = nullptr, *hd = nullptr;
    double* Vt = nullptr;  // ordinates scratch
    double* Vt2 = nullptr;
    // fully implicit step: adv_x transposed, D transposed, and the ordinates-space GMRES buffers
    // (allocated on first use)
    double *AxT = nullptr, *DT = nullptr;
    double *Fk = nullptr, *Fr = nullptr, *Fw = nullptr, *Fz = nullptr, *Fx = nullptr, *Fb = nullptr, *Ft = nullptr;
    double *Fpart = nullptr;
    int fcap = 0;
    std::vector<void*> allocs;
    long long launches = 0;
};

static thread_local std::string g_err1d;

#define CK1(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { g_err1d = std::string(#x) + ": " + cudaGetErrorString(_e); return BTE_ERR_CUDA; } } while (0)

// after the per-point FP32 block factorization: a zero pivot in any block is an error (its
// substitution would spread Inf/NaN into the step while GMRES could still report convergence)
static int check_blocks(Bte1d* h, cudaStream_t s) {
    std::vector<int32_t> info((size_t)h->Nx);
    CK1(cudaMemcpyAsync(info.data(), h->Vinfo, info.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK1(cudaStreamSynchronize(s));
    for (int x = 0; x < h->Nx; ++x)
        if (info[(size_t)x] != 0) {
            g_err1d = "singular v-space block at x point " + std::to_string(x) + " (zero pivot " +
                      std::to_string(info[(size_t)x]) + ")";
            return BTE_ERR_STATE;
        }
    return BTE_OK;
}

static int alloc1d(Bte1d* h, void** p, size_t bytes) {
    if (cudaMalloc(p, std::max<size_t>(bytes, 8)) != cudaSuccess) { g_err1d = "device allocation failed"; return BTE_ERR_ALLOC; }
    h->allocs.push_back(*p);
    return BTE_OK;
}

static void free1d(Bte1d* h) {
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
}

extern "C" {

const char* bte1d_last_error(void) { return g_err1d.c_str(); }

int bte1d_create(int device, int Nr, int nsh, int Nvt, int Nx, const double* Q, const double* Qinv, const double* d,
                 const double* cos_theta, const double* D, const double* po2sh, const double* psh2o,
                 const double* Cv, const double* Av, int restart, Bte1d** out) {
    if (!out || !Q || !Qinv || !d || !cos_theta || !D || !po2sh || !psh2o || !Cv || !Av) {
        g_err1d = "null argument";
        return BTE_ERR_ARG;
    }
    *out = nullptr;
    if (Nr < 4 || nsh < 1 || Nvt < 2 || (Nvt & 1) || Nx < 3 || Nx > 2048 || Nr * nsh > 512 || restart < 1 ||
        restart > 200) {
        g_err1d = "sizes out of range (Nr >= 4, Nvt even, 3 <= Nx <= 2048, Nr * nsh <= 512, 1 <= restart <= 200)";
        return BTE_ERR_ARG;
    }
    if (cudaSetDevice(device) != cudaSuccess) { g_err1d = "cudaSetDevice failed"; return BTE_ERR_CUDA; }
    Bte1d* h = new Bte1d();
    h->device = device; h->Nr = Nr; h->nsh = nsh; h->n = Nr * nsh; h->Nvt = Nvt; h->Nx = Nx; h->kcap = restart;
    const int n = h->n;
    const size_t nv = (size_t)Nr * Nvt * Nx, nu = (size_t)n * Nx;
    h->xld = (Nx + 3) & ~3;  // rows start on 16-byte boundaries (the LU kernels stage rows with cp.async)
    h->vld = (n + 3) & ~3;
    int rc = BTE_OK;
    auto A = [&](void** p, size_t b) { if (rc == BTE_OK) rc = alloc1d(h, p, b); };
    A((void**)&h->Q, (size_t)Nr * Nr * 8); A((void**)&h->Qinv, (size_t)Nr * Nr * 8); A((void**)&h->d, Nr * 8);
    A((void**)&h->cth, Nvt * 8); A((void**)&h->D, (size_t)Nx * Nx * 8); A((void**)&h->right, Nvt);
    A((void**)&h->Ps, (size_t)nsh * Nvt * 8); A((void**)&h->Po, (size_t)Nvt * nsh * 8);
    A((void**)&h->CvT, (size_t)n * n * 8); A((void**)&h->AvT, (size_t)n * n * 8);
    A((void**)&h->XA, (size_t)Nr * Nvt * Nx * h->xld * 8);
    A((void**)&h->XI, (size_t)Nr * Nvt * Nx * Nx * 8);
    A((void**)&h->Xpiv, (size_t)Nr * Nvt * Nx * 4); A((void**)&h->Xinfo, (size_t)Nr * Nvt * 4);
    A((void**)&h->VB, (size_t)Nx * n * h->vld * 4);
    A((void**)&h->Vpiv, (size_t)Nx * n * 4); A((void**)&h->Vinfo, (size_t)Nx * 4);
    A((void**)&h->U, nu * 8); A((void**)&h->R, nu * 8); A((void**)&h->W, nu * 8); A((void**)&h->Z, nu * 8);
    A((void**)&h->Xs, nu * 8); A((void**)&h->T, nu * 8); A((void**)&h->Zf, nu * 4);
    A((void**)&h->Kr, (size_t)(restart + 1) * nu * 8);
    A((void**)&h->part, (size_t)(restart + 1) * RED_BLOCKS * 8); A((void**)&h->hd, (size_t)(restart + 1) * 8);
    A((void**)&h->Vt, nv * 8);
    A((void**)&h->Vt2, nv * 8);
    A((void**)&h->AxT, (size_t)Nr * Nr * 8); A((void**)&h->DT, (size_t)Nx * Nx * 8);
    if (rc != BTE_OK) { free1d(h); delete h; return rc; }
    // adv_x = Q diag(d) Q^-1 (transposed), and D transposed, for the fully implicit step
    {
        std::vector<double> AxT((size_t)Nr * Nr), DT((size_t)Nx * Nx);
        for (int r = 0; r < Nr; ++r)
            for (int k = 0; k < Nr; ++k) {
                double v = 0.0;
                for (int i = 0; i < Nr; ++i) v += Q[(size_t)r * Nr + i] * d[i] * Qinv[(size_t)i * Nr + k];
                AxT[(size_t)k * Nr + r] = v;
            }
        for (int a = 0; a < Nx; ++a)
            for (int b = 0; b < Nx; ++b) DT[(size_t)b * Nx + a] = D[(size_t)a * Nx + b];
        if (cudaMemcpy(h->AxT, AxT.data(), AxT.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(h->DT, DT.data(), DT.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
            g_err1d = "copy of the setup operators failed";
            free1d(h);
            delete h;
            return BTE_ERR_CUDA;
        }
    }
    // transposed v-space operators; inflow side of each ordinate
    std::vector<double> CvT((size_t)n * n), AvT((size_t)n * n);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) { CvT[(size_t)b * n + a] = Cv[(size_t)a * n + b]; AvT[(size_t)b * n + a] = Av[(size_t)a * n + b]; }
    std::vector<int8_t> right(Nvt);
    for (int j = 0; j < Nvt; ++j) right[j] = cos_theta[j] >= 0.0 ? 1 : 0;
    bool ok = cudaMemcpy(h->Q, Q, (size_t)Nr * Nr * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->Qinv, Qinv, (size_t)Nr * Nr * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->d, d, Nr * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->cth, cos_theta, Nvt * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->D, D, (size_t)Nx * Nx * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->right, right.data(), Nvt, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->Ps, po2sh, (size_t)nsh * Nvt * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->Po, psh2o, (size_t)Nvt * nsh * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->CvT, CvT.data(), (size_t)n * n * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(h->AvT, AvT.data(), (size_t)n * n * 8, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) { g_err1d = "copy of the setup operators failed"; free1d(h); delete h; return BTE_ERR_CUDA; }
    *out = h;
    return BTE_OK;
}

int bte1d_destroy(Bte1d* h) {
    if (!h) return BTE_OK;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    free1d(h);
    delete h;
    return BTE_OK;
}

// x-advection over a step of size hstep (backward Euler); V in place (ordinates layout)
int bte1d_step_x(Bte1d* h, double hstep, double* V, void* stream) {
    if (!h || !V) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    const int Nr = h->Nr, Nvt = h->Nvt, Nx = h->Nx;
    const int C = Nvt * Nx;
    const long long xs = (long long)Nx * h->xld;
    if (hstep != h->hx) {  // factor I + h d_r cos(theta_j) D_X once per step size
        k_build_xshift<<<dim3(nb((size_t)Nx * Nx, 256) > 64 ? 64 : nb((size_t)Nx * Nx, 256), Nr * Nvt), 256, 0, s>>>(
            Nr, Nvt, Nx, hstep, h->d, h->cth, h->right, h->D, h->XA, h->xld, xs);
        CK1(cudaGetLastError());
        CK1(bte_lu_factor_t<double>(Nr * Nvt, Nx, Nx, h->XA, h->xld, xs, h->Xpiv, h->Xinfo, s, 0));
        std::vector<int32_t> info(Nr * Nvt);
        CK1(cudaMemcpyAsync(info.data(), h->Xinfo, info.size() * 4, cudaMemcpyDeviceToHost, s));
        CK1(cudaStreamSynchronize(s));
        for (int v : info)
            if (v != 0) { g_err1d = "x-advection matrix is singular"; return BTE_ERR_STATE; }
        // explicit inverses, one identity column per pass (as the reference applies them,
        // :780-887): each step then streams them once, an HBM-bound batched product
        const int P = Nr * Nvt;
        for (int c = 0; c < Nx; ++c) {
            k_unit_rhs<<<nb((size_t)P * Nx, 256), 256, 0, s>>>(P, Nx, c, h->Vt);
            CK1(bte_lu_solve_t<double>(P, Nx, h->XA, h->xld, xs, h->Xpiv, h->Vt, 0, s));
            k_store_invcol<<<nb((size_t)P * Nx, 256), 256, 0, s>>>(P, Nx, c, h->Vt, h->XI);
        }
        CK1(cudaGetLastError());
        h->hx = hstep;
        h->launches += 2 + 3 * (long long)Nx;
    }
    const size_t smem = (size_t)Nr * Nr * 8;
    CK1(bte_raise_smem_limit((const void*)k_radial_mix, smem));
    k_radial_mix<<<dim3(nb(C, 128), Nr), 128, smem, s>>>(Nr, C, h->Qinv, V, h->Vt);
    k_zero_inflow<<<nb((size_t)Nr * Nvt, 256), 256, 0, s>>>(Nr, Nvt, Nx, h->right, h->Vt);
    CK1(cudaGetLastError());
    k_xstep_apply<<<Nr * Nvt, 256, (size_t)Nx * 8, s>>>(Nx, h->XI, h->Vt, h->Vt2);
    k_radial_mix<<<dim3(nb(C, 128), Nr), 128, smem, s>>>(Nr, C, h->Q, h->Vt2, V);
    CK1(cudaGetLastError());
    h->launches += 4;
    return BTE_OK;
}

// Lmat_mvec in the x-major v-space layout (for tests and for callers with their own solver)
int bte1d_lmat(Bte1d* h, double dt, const double* E, const double* X, double* Y, void* stream) {
    if (!h || !E || !X || !Y) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    const size_t smem = (size_t)MV_X * h->n * 8;
    k_lmat<<<nb(h->Nx, MV_X), 128, smem, (cudaStream_t)stream>>>(h->n, h->Nx, dt, h->CvT, h->AvT, E, X, Y);
    CK1(cudaGetLastError());
    h->launches += 1;
    return BTE_OK;
}

// v-space step: V (ordinates) in place. info4 (host) = {GMRES iterations, ||b - A x||,
// ||b - A x|| / ||b||, 0 converged / 1 not}.
int bte1d_step_v(Bte1d* h, double dt, const double* E, double* V, double rtol, double atol, int max_iter,
                 double* info4, void* stream) {
    if (!h || !E || !V || !info4) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    const int n = h->n, Nx = h->Nx, m = h->kcap;
    const size_t N = (size_t)n * Nx;
    const long long vs = (long long)n * h->vld;
    long long L = 0;
    auto lmat = [&](const double* x, double* y) {
        k_lmat<<<nb(Nx, MV_X), 128, (size_t)MV_X * n * 8, s>>>(n, Nx, dt, h->CvT, h->AvT, E, x, y);
        ++L;
    };
    auto precond = [&](const double* x, double* y) -> cudaError_t {  // y = M^-1 x (per-x FP32 block LU)
        k_to_f32<<<nb(N, 256), 256, 0, s>>>(N, x, h->Zf);
        cudaError_t e = bte_lu_solve_t<float>(Nx, n, h->VB, h->vld, vs, h->Vpiv, h->Zf, 0, s);
        k_to_f64<<<nb(N, 256), 256, 0, s>>>(N, h->Zf, y);
        L += 3;
        return e;
    };
    auto dots = [&](int k, const double* Vb, const double* w, double* host_out) -> cudaError_t {
        k_dots_partial<<<dim3(RED_BLOCKS, k), 256, 0, s>>>(N, k, Vb, N, w, h->part);
        k_dots_final<<<k, 256, 0, s>>>(k, RED_BLOCKS, h->part, h->hd);
        L += 2;
        cudaError_t e = cudaMemcpyAsync(host_out, h->hd, k * 8, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return e;
        return cudaStreamSynchronize(s);
    };
    // right-hand side U = P_o2sh V, and the per-point FP32 block factors
    k_ords_to_lm<<<nb(N, 256), 256, 0, s>>>(h->Nr, h->Nvt, h->nsh, Nx, h->Ps, V, h->U);
    k_build_vblocks<<<dim3(std::min<unsigned>(nb((size_t)n * n, 256), 32), Nx), 256, 0, s>>>(n, Nx, dt, h->CvT, h->AvT, E,
                                                                                        h->VB, h->vld, vs);
    CK1(cudaGetLastError());
    CK1(bte_lu_factor_t<float>(Nx, n, n, h->VB, h->vld, vs, h->Vpiv, h->Vinfo, s, 0));
    L += 3;
    if (int rc = check_blocks(h, s)) return rc;
    double bnorm = 0.0;
    CK1(dots(1, h->U, h->U, &bnorm));
    bnorm = std::sqrt(bnorm);
    const double tol = std::max(atol, rtol * bnorm);
    // x0 = M^-1 b
    CK1(precond(h->U, h->Xs));
    int it = 0;
    double rnorm = 0.0;
    bool conv = false;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hh(m + 1), y(m);
    while (true) {
        lmat(h->Xs, h->W);
        k_sub<<<nb(N, 256), 256, 0, s>>>(N, h->U, h->W, h->R);
        ++L;
        CK1(dots(1, h->R, h->R, &rnorm));
        rnorm = std::sqrt(rnorm);
        if (rnorm <= tol) { conv = true; break; }
        if (it >= max_iter) break;
        k_scale<<<nb(N, 256), 256, 0, s>>>(N, 1.0 / rnorm, h->R, h->Kr);
        ++L;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = rnorm;
        int k = 0;
        for (; k < m && it < max_iter; ++k, ++it) {
            double* vk = h->Kr + (size_t)k * N;
            double* vk1 = h->Kr + (size_t)(k + 1) * N;
            CK1(precond(vk, h->Z));
            lmat(h->Z, vk1);
            // classical Gram-Schmidt, applied twice
            for (int pass = 0; pass < 2; ++pass) {
                CK1(dots(k + 1, h->Kr, vk1, hh.data()));
                CK1(cudaMemcpyAsync(h->hd, hh.data(), (k + 1) * 8, cudaMemcpyHostToDevice, s));
                k_sub_combo<<<nb(N, 256), 256, 0, s>>>(N, k + 1, h->Kr, N, h->hd, vk1);
                ++L;
                for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = (pass == 0 ? 0.0 : H[(size_t)j * m + k]) + hh[j];
            }
            double nn = 0.0;
            CK1(dots(1, vk1, vk1, &nn));
            nn = std::sqrt(nn);
            H[(size_t)(k + 1) * m + k] = nn;
            if (nn > 0) { k_scale<<<nb(N, 256), 256, 0, s>>>(N, 1.0 / nn, vk1, vk1); ++L; }
            // Givens rotations on column k
            for (int j = 0; j < k; ++j) {
                const double a = H[(size_t)j * m + k], b = H[(size_t)(j + 1) * m + k];
                H[(size_t)j * m + k] = cs[j] * a + sn[j] * b;
                H[(size_t)(j + 1) * m + k] = -sn[j] * a + cs[j] * b;
            }
            const double a = H[(size_t)k * m + k], b = H[(size_t)(k + 1) * m + k];
            const double rr = std::hypot(a, b);
            cs[k] = rr > 0 ? a / rr : 1.0;
            sn[k] = rr > 0 ? b / rr : 0.0;
            H[(size_t)k * m + k] = rr;
            H[(size_t)(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            if (std::fabs(g[k + 1]) <= tol || nn == 0.0) { ++k; ++it; break; }
        }
        // y = H^-1 g (upper triangular k x k), x += M^-1 (V y)
        for (int i = k - 1; i >= 0; --i) {
            double acc = g[i];
            for (int j = i + 1; j < k; ++j) acc -= H[(size_t)i * m + j] * y[j];
            y[i] = H[(size_t)i * m + i] != 0.0 ? acc / H[(size_t)i * m + i] : 0.0;  // Krylov breakdown
        }
        CK1(cudaMemcpyAsync(h->hd, y.data(), k * 8, cudaMemcpyHostToDevice, s));
        k_combo<<<nb(N, 256), 256, 0, s>>>(N, k, h->Kr, N, h->hd, h->T);
        ++L;
        CK1(precond(h->T, h->Z));
        k_axpy<<<nb(N, 256), 256, 0, s>>>(N, 1.0, h->Z, h->Xs);
        ++L;
    }
    k_lm_to_ords<<<nb((size_t)h->Nr * h->Nvt * Nx, 256), 256, 0, s>>>(h->Nr, h->Nvt, h->nsh, Nx, h->Po, h->Xs, V);
    CK1(cudaGetLastError());
    CK1(cudaStreamSynchronize(s));
    h->launches += L + 1;
    info4[0] = it;
    info4[1] = rnorm;
    info4[2] = bnorm > 0 ? rnorm / bnorm : 0.0;
    info4[3] = conv ? 0.0 : 1.0;
    return BTE_OK;
}

// Block preconditioner: factor each point's block I - dt (Cv + E_x Av) in FP32 and apply its
// inverse to X (x-major v-space layout) -> Y, in FP64 storage
int bte1d_block_solve(Bte1d* h, double dt, const double* E, const double* X, double* Y, void* stream) {
    if (!h || !E || !X || !Y) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    const int n = h->n, Nx = h->Nx;
    const size_t N = (size_t)n * Nx;
    const long long vs = (long long)n * h->vld;
    k_build_vblocks<<<dim3(std::min<unsigned>(nb((size_t)n * n, 256), 32), Nx), 256, 0, s>>>(n, Nx, dt, h->CvT, h->AvT, E,
                                                                                        h->VB, h->vld, vs);
    CK1(cudaGetLastError());
    CK1(bte_lu_factor_t<float>(Nx, n, n, h->VB, h->vld, vs, h->Vpiv, h->Vinfo, s, 0));
    if (int rc = check_blocks(h, s)) return rc;
    k_to_f32<<<nb(N, 256), 256, 0, s>>>(N, X, h->Zf);
    CK1(bte_lu_solve_t<float>(Nx, n, h->VB, h->vld, vs, h->Vpiv, h->Zf, 0, s));
    k_to_f64<<<nb(N, 256), 256, 0, s>>>(N, h->Zf, Y);
    CK1(cudaGetLastError());
    h->launches += 5;
    return BTE_OK;
}

// ordinates <-> spherical harmonics (ords_to_sph / sph_to_ords, bte_1d3v_solver.py:678-694) in
// the x-major v-space layout
int bte1d_ords_to_lm(Bte1d* h, const double* V, double* U, void* stream) {
    if (!h || !V || !U) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    k_ords_to_lm<<<nb((size_t)h->n * h->Nx, 256), 256, 0, (cudaStream_t)stream>>>(h->Nr, h->Nvt, h->nsh, h->Nx, h->Ps, V, U);
    CK1(cudaGetLastError());
    return BTE_OK;
}
int bte1d_lm_to_ords(Bte1d* h, const double* U, double* V, void* stream) {
    if (!h || !V || !U) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    k_lm_to_ords<<<nb((size_t)h->Nr * h->Nvt * h->Nx, 256), 256, 0, (cudaStream_t)stream>>>(h->Nr, h->Nvt, h->nsh, h->Nx,
                                                                                            h->Po, U, V);
    CK1(cudaGetLastError());
    return BTE_OK;
}

// ---- fully implicit spectral step ------------------------------------------------------------
static int fim_matvec(Bte1d* h, double dt, const double* E, const double* V, double* Y, cudaStream_t s) {
    const int Nr = h->Nr, Nvt = h->Nvt, Nx = h->Nx, M = Nr * Nvt;
    if (!h->Ft && alloc1d(h, (void**)&h->Ft, (size_t)M * Nx * 8) != BTE_OK) return BTE_ERR_ALLOC;
    const size_t sdx = (size_t)FD_L * Nx * 8;
    const size_t scb = ((size_t)2 * FC_X * M + 2 * FC_X * h->n + (size_t)Nr * Nr) * 8;
    CK1(bte_raise_smem_limit((const void*)k_fim_dx, sdx));
    CK1(bte_raise_smem_limit((const void*)k_fim_combine, scb));
    k_fim_dx<<<nb(M, FD_L), 256, sdx, s>>>(M, Nvt, Nx, h->DT, h->right, V, h->Ft);
    k_fim_combine<<<nb(Nx, FC_X), 256, scb, s>>>(Nr, Nvt, h->nsh, Nx, dt, h->Ps, h->Po, h->CvT, h->AvT, h->AxT,
                                                 h->cth, h->right, E, V, h->Ft, Y);
    CK1(cudaGetLastError());
    h->launches += 2;
    return BTE_OK;
}

int bte1d_fim_matvec(Bte1d* h, double dt, const double* E, const double* V, double* Y, void* stream) {
    if (!h || !E || !V || !Y) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    return fim_matvec(h, dt, E, V, Y, (cudaStream_t)stream);
}

int bte1d_step_fim(Bte1d* h, double dt, const double* E, double* V, double rtol, double atol, int max_iter, int pc,
                   double* info4, void* stream) {
    if (!h || !E || !V || !info4) { g_err1d = "null argument"; return BTE_ERR_ARG; }
    if (pc < 0 || pc > 1 || max_iter < 1) { g_err1d = "pc must be 0 (split) or 1 (v-blocks); max_iter >= 1"; return BTE_ERR_ARG; }
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    const int Nr = h->Nr, Nvt = h->Nvt, Nx = h->Nx, n = h->n, m = h->kcap;
    const size_t N = (size_t)Nr * Nvt * Nx, Nu = (size_t)n * Nx;
    const long long vs = (long long)n * h->vld;
    if (h->fcap == 0) {
        int rc = BTE_OK;
        auto A = [&](void** p, size_t b) { if (rc == BTE_OK) rc = alloc1d(h, p, b); };
        A((void**)&h->Fk, (size_t)(m + 1) * N * 8);
        A((void**)&h->Fr, N * 8); A((void**)&h->Fw, N * 8); A((void**)&h->Fz, N * 8); A((void**)&h->Fx, N * 8);
        A((void**)&h->Fb, N * 8);
        A((void**)&h->Fpart, (size_t)(m + 1) * RED_BLOCKS * 8);
        if (rc != BTE_OK) return rc;
        h->fcap = m;
    }
    long long L = 0;
    // the per-point FP32 blocks I - dt (Cv + E_x Av) of the preconditioner's v part
    k_build_vblocks<<<dim3(std::min<unsigned>(nb((size_t)n * n, 256), 32), Nx), 256, 0, s>>>(n, Nx, dt, h->CvT, h->AvT, E,
                                                                                        h->VB, h->vld, vs);
    CK1(cudaGetLastError());
    CK1(bte_lu_factor_t<float>(Nx, n, n, h->VB, h->vld, vs, h->Vpiv, h->Vinfo, s, 0));
    L += 2;
    if (int rc = check_blocks(h, s)) return rc;
    auto precond = [&](const double* x, double* y) -> int {
        // v part: y = x + P_sh2o ((I - dt L_v)^-1 - I) P_o2sh x, per point, FP32 factors
        k_ords_to_lm<<<nb(Nu, 256), 256, 0, s>>>(Nr, Nvt, h->nsh, Nx, h->Ps, x, h->U);
        k_to_f32<<<nb(Nu, 256), 256, 0, s>>>(Nu, h->U, h->Zf);
        CK1(bte_lu_solve_t<float>(Nx, n, h->VB, h->vld, vs, h->Vpiv, h->Zf, 0, s));
        k_to_f64<<<nb(Nu, 256), 256, 0, s>>>(Nu, h->Zf, h->Z);
        k_lm_correct<<<nb(N, 256), 256, 0, s>>>(Nr, Nvt, h->nsh, Nx, h->Po, x, h->Z, h->U, y);
        CK1(cudaGetLastError());
        L += 5;
        // x part (pc 0): the backward-Euler x-advection over dt
        if (pc == 0) {
            int rc = bte1d_step_x(h, dt, y, s);
            if (rc) return rc;
        }
        return BTE_OK;
    };
    auto dots = [&](int k, const double* Vb, const double* w, double* host_out) -> cudaError_t {
        k_dots_partial<<<dim3(RED_BLOCKS, k), 256, 0, s>>>(N, k, Vb, N, w, h->Fpart);
        k_dots_final<<<k, 256, 0, s>>>(k, RED_BLOCKS, h->Fpart, h->hd);
        L += 2;
        cudaError_t e = cudaMemcpyAsync(host_out, h->hd, k * 8, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return e;
        return cudaStreamSynchronize(s);
    };
    // b = V with the inflow values set to 0 (the boundary condition); x0 = P^-1 b
    k_copy_zero_inflow<<<nb(N, 256), 256, 0, s>>>(Nr, Nvt, Nx, h->right, V, h->Fb);
    ++L;
    double bnorm = 0.0;
    CK1(dots(1, h->Fb, h->Fb, &bnorm));
    bnorm = std::sqrt(bnorm);
    const double tol = std::max(atol, rtol * bnorm);
    if (int rc = precond(h->Fb, h->Fx)) return rc;
    int it = 0;
    double rnorm = 0.0;
    bool conv = false;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hh(m + 1), y(m);
    while (true) {
        if (int rc = fim_matvec(h, dt, E, h->Fx, h->Fw, s)) return rc;
        k_sub<<<nb(N, 256), 256, 0, s>>>(N, h->Fb, h->Fw, h->Fr);
        ++L;
        CK1(dots(1, h->Fr, h->Fr, &rnorm));
        rnorm = std::sqrt(rnorm);
        if (rnorm <= tol) { conv = true; break; }
        if (it >= max_iter) break;
        k_scale<<<nb(N, 256), 256, 0, s>>>(N, 1.0 / rnorm, h->Fr, h->Fk);
        ++L;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = rnorm;
        int k = 0;
        for (; k < m && it < max_iter; ++k, ++it) {
            double* vk = h->Fk + (size_t)k * N;
            double* vk1 = h->Fk + (size_t)(k + 1) * N;
            if (int rc = precond(vk, h->Fz)) return rc;
            if (int rc = fim_matvec(h, dt, E, h->Fz, vk1, s)) return rc;
            for (int pass = 0; pass < 2; ++pass) {  // classical Gram-Schmidt, applied twice
                CK1(dots(k + 1, h->Fk, vk1, hh.data()));
                CK1(cudaMemcpyAsync(h->hd, hh.data(), (k + 1) * 8, cudaMemcpyHostToDevice, s));
                k_sub_combo<<<nb(N, 256), 256, 0, s>>>(N, k + 1, h->Fk, N, h->hd, vk1);
                ++L;
                for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = (pass == 0 ? 0.0 : H[(size_t)j * m + k]) + hh[j];
            }
            double nn = 0.0;
            CK1(dots(1, vk1, vk1, &nn));
            nn = std::sqrt(nn);
            H[(size_t)(k + 1) * m + k] = nn;
            if (nn > 0) { k_scale<<<nb(N, 256), 256, 0, s>>>(N, 1.0 / nn, vk1, vk1); ++L; }
            for (int j = 0; j < k; ++j) {  // Givens rotations on column k
                const double a = H[(size_t)j * m + k], b = H[(size_t)(j + 1) * m + k];
                H[(size_t)j * m + k] = cs[j] * a + sn[j] * b;
                H[(size_t)(j + 1) * m + k] = -sn[j] * a + cs[j] * b;
            }
            const double a = H[(size_t)k * m + k], b = H[(size_t)(k + 1) * m + k];
            const double rr = std::hypot(a, b);
            cs[k] = rr > 0 ? a / rr : 1.0;
            sn[k] = rr > 0 ? b / rr : 0.0;
            H[(size_t)k * m + k] = rr;
            H[(size_t)(k + 1) * m + k] = 0.0;
            g[k + 1] = -sn[k] * g[k];
            g[k] = cs[k] * g[k];
            if (std::fabs(g[k + 1]) <= tol || nn == 0.0) { ++k; ++it; break; }
        }
        for (int i = k - 1; i >= 0; --i) {  // y = H^-1 g, then x += P^-1 (V y)
            double acc = g[i];
            for (int j = i + 1; j < k; ++j) acc -= H[(size_t)i * m + j] * y[j];
            y[i] = H[(size_t)i * m + i] != 0.0 ? acc / H[(size_t)i * m + i] : 0.0;
        }
        CK1(cudaMemcpyAsync(h->hd, y.data(), k * 8, cudaMemcpyHostToDevice, s));
        k_combo<<<nb(N, 256), 256, 0, s>>>(N, k, h->Fk, N, h->hd, h->Fr);
        ++L;
        if (int rc = precond(h->Fr, h->Fz)) return rc;
        k_axpy<<<nb(N, 256), 256, 0, s>>>(N, 1.0, h->Fz, h->Fx);
        ++L;
    }
    CK1(cudaMemcpyAsync(V, h->Fx, N * 8, cudaMemcpyDeviceToDevice, s));
    CK1(cudaStreamSynchronize(s));
    h->launches += L;
    info4[0] = it;
    info4[1] = rnorm;
    info4[2] = bnorm > 0 ? rnorm / bnorm : 0.0;
    info4[3] = conv ? 0.0 : 1.0;
    return BTE_OK;
}

long long bte1d_launches(const Bte1d* h) { return h ? h->launches : 0; }


}  // extern "C"
