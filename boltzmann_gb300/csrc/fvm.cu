// Finite-volume 1D3V fully implicit step on the GPU (sm_103a): the reference's
// solver_type "fully_implicit" (bte_1d3v_solver.py:1890-2009), preconditioned by its op-split
// step (:1745-1870, type XVTVRC).
//
// Operator: one fused kernel (k_fvm_mvec, fvm_core.h) reads each value's upwind stencils along
// x, v_r and v_theta and writes one output, after the ordinate moments m = w^T v
// (k_fvm_moment) and the gain product G m (FP64 GEMM, Nr x Nr by Nr x Nx). The reference
// multiplies dense (Nr Nvt)^2 collision and advection matrices instead; here the work per
// value is O(p + Nr), so the operator is one read and one write of v (HBM-bound).
// Preconditioner: the collision inverse in closed form, (D^-1 (x) I + H (x) 1 w^T) v, then the
// v_r, v_theta and x sweeps in the natural layout: the v_r and v_theta recurrences run one
// thread per line with the warp's lanes on consecutive x (coalesced), the x recurrence on rows
// staged in shared memory; the reference (and the drop-in sweeps of sweeps.cu) swap layouts
// between the sweeps instead.
// Solver: restarted right-preconditioned GMRES (fvm_core.h), device vectors, FP64.
// Semi-Lagrangian step (solver_type "sl_implicit", :2024-2027): one kernel interpolates every
// value at its departure point (k_fvm_sl), then the closed-form collision inverse.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <vector>

#include "bte_common.cuh"
#include "fvm_core.h"
#include "../../include/bte_fvm_gb300.h"
#include "../../include/bte_sweeps_gb300.h"

struct bte_fvm {
    int device = 0;
    int Nr = 0, Nvt = 0, Nx = 0, ndr = 0, ndt = 0, ndx = 0;
    size_t N = 0;
    double *vr = nullptr, *vt = nullptr, *cos_t = nullptr, *w = nullptr, *loss = nullptr, *gain = nullptr;
    int8_t* north = nullptr;
    double *vrL = nullptr, *vrR = nullptr, *vtL = nullptr, *vtR = nullptr, *xL = nullptr, *xR = nullptr;
    double *dinv = nullptr, *H = nullptr;   // collision inverse factors (set per step size)
    bool have_inverse = false;
    double *M = nullptr, *T = nullptr, *aE = nullptr, *axvr = nullptr;   // (Nr, Nx), (Nr, Nx), Nx, Nr
    double *A = nullptr, *Bf = nullptr;                                  // N each
    double *B = nullptr, *X = nullptr, *R = nullptr, *W = nullptr, *Z = nullptr, *Tv = nullptr;
    double* Kr = nullptr;
    int kcap = 0;
    double *part = nullptr, *hd = nullptr;
    double *xg = nullptr, *vrp = nullptr, *vta = nullptr;   // semi-Lagrangian grids (set once)
    double sl_vmin = 0.0;
    bool have_sl = false;
    std::vector<void*> allocs;
    long long launches = 0;
};

namespace {

constexpr int FT = 256;          // threads of the element kernels
constexpr int FVM_RED = 120;     // partial-sum blocks of the reductions (fixed: deterministic order)

thread_local std::string g_fvm_err;

int fvm_fail(int code, const std::string& msg) {
    g_fvm_err = msg;
    return code;
}

inline unsigned fblocks(size_t n) { return (unsigned)((n + FT - 1) / FT); }

FvmView view_of(const bte_fvm* h) {
    FvmView v;
    v.Nr = h->Nr; v.Nvt = h->Nvt; v.Nx = h->Nx;
    v.ndr = h->ndr; v.ndt = h->ndt; v.ndx = h->ndx;
    v.vr = h->vr; v.cos_t = h->cos_t; v.north = h->north; v.w = h->w; v.loss = h->loss;
    v.vrL = h->vrL; v.vrR = h->vrR; v.vtL = h->vtL; v.vtR = h->vtR; v.xL = h->xL; v.xR = h->xR;
    return v;
}

// m[r][x] = sum_j w_j X[r][j][x], one thread per (r, x)
__global__ void k_fvm_moment(FvmView v, const double* __restrict__ X, double* __restrict__ m) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)v.Nr * v.Nx) return;
    const int x = (int)(i % v.Nx), r = (int)(i / v.Nx);
    m[i] = fvm_moment_at(v, X, r, x);
}

// Y = rhs_mvec(X), one thread per value, x fastest
__global__ void k_fvm_mvec(FvmView v, FvmCoef c, const double* __restrict__ E, const double* __restrict__ G,
                           const double* __restrict__ X, double* __restrict__ Y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)v.Nr * v.Nvt * v.Nx;
    if (i >= n) return;
    const int x = (int)(i % v.Nx);
    const size_t rj = i / v.Nx;
    const int j = (int)(rj % v.Nvt), r = (int)(rj / v.Nvt);
    Y[i] = fvm_mvec_at(v, c, E, G, X, r, j, x);
}

// out (Nx, Nvt, Nr) = the collision inverse applied to B (Nr, Nvt, Nx), one thread per output
__global__ void k_fvm_coll_permute(FvmView v, const double* __restrict__ dinv, const double* __restrict__ T,
                                   const double* __restrict__ B, double* __restrict__ out) {
    const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)v.Nr * v.Nvt * v.Nx;
    if (o >= n) return;
    const int r = (int)(o % v.Nr);
    const size_t xj = o / v.Nr;
    const int j = (int)(xj % v.Nvt), x = (int)(xj / v.Nvt);
    out[o] = fvm_coll_apply_at(v, dinv, T, B, r, j, x);
}

// Y (Nr, Nvt, Nx) = the collision inverse applied to B, same layout
__global__ void k_fvm_coll_apply(FvmView v, const double* __restrict__ dinv, const double* __restrict__ T,
                                 const double* __restrict__ B, double* __restrict__ Y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)v.Nr * v.Nvt * v.Nx;
    if (i >= n) return;
    const int x = (int)(i % v.Nx);
    const size_t rj = i / v.Nx;
    Y[i] = fvm_coll_apply_at(v, dinv, T, B, (int)(rj / v.Nvt), (int)(rj % v.Nvt), x);
}

// Y = the semi-Lagrangian advection of V, one thread per value
// ---- preconditioner sweeps in the natural (Nr, Nvt, Nx) layout --------------------------------
// One upwind backward-Euler recurrence (I + a h D) o = b per thread along a line of N values
// spaced `stride` apart, in place. The bands are the sweeps' column-stored ones (lower
// D[i][i-k] = L[k][i-k], upper D[i][i+k] = R[k][i+k], rawkernel.py:168-375); the last nd - 1
// outputs of the line stay in registers. Along v_r (stride Nvt Nx) and v_theta (stride Nx)
// the threads of a warp take consecutive x, so every step is one coalesced 256-byte access:
// no layout swaps, unlike the reference's sweeps on permuted copies. L and R are the calling
// CTA's shared-memory copies of the bands (stage_bands), so a step waits on no global load but
// its right-hand side, which is loaded SW_PF steps ahead.
constexpr int SW_NDMAX = 4;
constexpr int SW_PF = 8;   // right-hand sides loaded ahead of the recurrence
__device__ inline void stage_bands(const double* __restrict__ L, const double* __restrict__ R, int nd, int N,
                                   double* sL, double* sR) {
    for (int e = threadIdx.x; e < nd * N; e += blockDim.x) {
        sL[e] = L[e];
        sR[e] = R[e];
    }
}
// With rc (the reciprocals of the line's diagonal 1 + ad D[i][i], at the same positions as v,
// k_fvm_diag_rcp) a step is five FP64 operations instead of a division's dozen: the few long
// v_r and x lines run one warp per SM, each bound by its SM sub-partition's FP64 issue rate.
template <bool RC>
__device__ inline void fvm_sweep_line(const double* L, const double* R, int nd, int N,
                                      double ad, bool ltr, double* __restrict__ v, long long stride,
                                      const double* __restrict__ rc = nullptr) {
    double prev[SW_NDMAX - 1];
#pragma unroll
    for (int k = 0; k < SW_NDMAX - 1; ++k) prev[k] = 0.0;
    const double* B = ltr ? L : R;
    // the loads of b (and of the reciprocals) do not depend on the recurrence: keep SW_PF of
    // them in flight
    double pf[SW_PF], pr[SW_PF];
#pragma unroll
    for (int q = 0; q < SW_PF; ++q) {
        const long long o = (long long)(ltr ? q : N - 1 - q) * stride;
        pf[q] = (q < N) ? v[o] : 0.0;
        if (RC) pr[q] = (q < N) ? rc[o] : 0.0;
    }
    for (int step = 0; step < N; ++step) {
        const int i = ltr ? step : N - 1 - step;
        const double bi = pf[0];
        const double ri = RC ? pr[0] : 0.0;
#pragma unroll
        for (int q = 0; q < SW_PF - 1; ++q) {
            pf[q] = pf[q + 1];
            if (RC) pr[q] = pr[q + 1];
        }
        const int nxt = step + SW_PF;
        const long long on = (long long)(ltr ? nxt : N - 1 - nxt) * stride;
        pf[SW_PF - 1] = (nxt < N) ? v[on] : 0.0;
        if (RC) pr[SW_PF - 1] = (nxt < N) ? rc[on] : 0.0;
        double sacc = 0.0;
#pragma unroll
        for (int k = 1; k < SW_NDMAX; ++k)
            if (k < nd && step >= k) sacc += B[(size_t)k * N + (ltr ? i - k : i + k)] * prev[k - 1];
        const double o = RC ? (bi - ad * sacc) * ri : (bi - ad * sacc) / (1.0 + ad * B[i]);
#pragma unroll
        for (int k = SW_NDMAX - 2; k > 0; --k) prev[k] = prev[k - 1];
        prev[0] = o;
        v[(long long)i * stride] = o;
    }
}

// Rc = 1 / (1 + a h D[i][i]) at every position of the natural layout, for the v_r sweep
// (which = 0: a and the band as k_fvm_sweep_vr takes them, i = r) or the x sweep (which = 2:
// as k_fvm_sweep_x, i = x); all SMs share the divisions the recurrences would serialise
__global__ void k_fvm_diag_rcp(FvmView v, int which, const double* __restrict__ aE,
                               const double* __restrict__ axvr, double h, double* __restrict__ Rc) {
    const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)v.Nr * v.Nvt * v.Nx;
    if (o >= n) return;
    const int x = (int)(o % v.Nx);
    const size_t rj = o / v.Nx;
    const int j = (int)(rj % v.Nvt), r = (int)(rj / v.Nvt);
    double a, d;
    if (which == 0) {
        a = -aE[x] * v.cos_t[j];
        d = (a >= 0.0 ? v.vrL : v.vrR)[r];
    } else {
        a = axvr[r] * v.cos_t[j];
        d = (a >= 0.0 ? v.xL : v.xR)[x];
    }
    const double ad = a * h;
    Rc[o] = 1.0 / (1.0 + ad * d);
}

// v_r sweep: line (j, x), a = -aE[x] cos(theta_j), left to right when a >= 0 (rawkernel.py:168-230)
__global__ void k_fvm_sweep_vr(FvmView v, const double* __restrict__ aE, double h, double* __restrict__ V,
                               const double* __restrict__ Rc) {
    extern __shared__ double sband[];  // [2][ndr][Nr]
    double *sL = sband, *sR = sband + (size_t)v.ndr * v.Nr;
    stage_bands(v.vrL, v.vrR, v.ndr, v.Nr, sL, sR);
    __syncthreads();
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= v.Nvt * v.Nx) return;
    const int j = line / v.Nx, x = line % v.Nx;
    const double a = -aE[x] * v.cos_t[j];
    fvm_sweep_line<true>(sL, sR, v.ndr, v.Nr, a * h, a >= 0.0, V + (size_t)j * v.Nx + x, (long long)v.Nvt * v.Nx,
                         Rc + (size_t)j * v.Nx + x);
}

// v_theta sweep: line (r, x), a = aE[x] / v_r, left to right when -a >= 0 (rawkernel.py:232-296)
__global__ void k_fvm_sweep_vt(FvmView v, const double* __restrict__ aE, double h, double* __restrict__ V) {
    extern __shared__ double sband[];  // [2][ndt][Nvt]
    double *sL = sband, *sR = sband + (size_t)v.ndt * v.Nvt;
    stage_bands(v.vtL, v.vtR, v.ndt, v.Nvt, sL, sR);
    __syncthreads();
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= v.Nr * v.Nx) return;
    const int r = line / v.Nx, x = line % v.Nx;
    const double a = aE[x] / v.vr[r];
    fvm_sweep_line<false>(sL, sR, v.ndt, v.Nvt, a * h, -a >= 0.0, V + (size_t)r * v.Nvt * v.Nx + x, (long long)v.Nx);
}

// x sweep with the inflow values zeroed first: line (r, j) is a contiguous row of Nx values;
// a CTA stages XT_L consecutive rows (one contiguous block) in shared memory with coalesced
// loads, sweeps each row in shared memory (row pitch Nx + 1 against bank conflicts) and
// writes the block back coalesced. a = ax v_r cos(theta_j), left to right when a >= 0
// (rawkernel.py:298-375).
constexpr int XT_L = 32;       // rows per CTA
constexpr int XT_T = 256;      // threads per CTA: all load and store, the first XT_L sweep
__global__ void __launch_bounds__(XT_T) k_fvm_sweep_x(FvmView v, const double* __restrict__ axvr, double h,
                                                      const double* __restrict__ B, double* __restrict__ Y,
                                                      const double* __restrict__ Rc) {
    extern __shared__ double rows[];  // [XT_L][Nx + 1], then the bands [2][ndx][Nx]
    const int Nx = v.Nx, pitch = Nx + 1;
    double* sL = rows + (size_t)XT_L * pitch;
    double* sR = sL + (size_t)v.ndx * Nx;
    stage_bands(v.xL, v.xR, v.ndx, Nx, sL, sR);
    const int nlines = v.Nr * v.Nvt;
    const int l0 = blockIdx.x * XT_L;
    const int nl = min(XT_L, nlines - l0);
    const double* src = B + (size_t)l0 * Nx;
    for (int e = threadIdx.x; e < nl * Nx; e += blockDim.x) {
        const int l = e / Nx, x = e % Nx;
        const int j = (l0 + l) % v.Nvt;
        const bool inflow = v.north[j] ? (x == 0) : (x == Nx - 1);
        rows[l * pitch + x] = inflow ? 0.0 : src[e];
    }
    __syncthreads();
    if (threadIdx.x < nl) {
        const int line = l0 + threadIdx.x;
        const int r = line / v.Nvt, j = line % v.Nvt;
        const double a = axvr[r] * v.cos_t[j];
        fvm_sweep_line<true>(sL, sR, v.ndx, Nx, a * h, a >= 0.0, rows + threadIdx.x * pitch, 1,
                             Rc + (size_t)line * Nx);
    }
    __syncthreads();
    double* dst = Y + (size_t)l0 * Nx;
    for (int e = threadIdx.x; e < nl * Nx; e += blockDim.x) dst[e] = rows[(e / Nx) * pitch + e % Nx];
}

__global__ void k_fvm_sl(FvmSl sl, const double* __restrict__ E, const double* __restrict__ V, double* __restrict__ Y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)sl.Nr * sl.Nvt * sl.Nx;
    if (i >= n) return;
    const int x = (int)(i % sl.Nx);
    const size_t rj = i / sl.Nx;
    Y[i] = fvm_sl_at(sl, E, V, (int)(rj / sl.Nvt), (int)(rj % sl.Nvt), x);
}

// y = a x (x may alias y)
__global__ void k_fvm_scale(size_t n, double a, const double* x, double* y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i];
}
__global__ void k_fvm_axpy(size_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}
__global__ void k_fvm_sub(size_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) c[i] = a[i] - b[i];
}
// w -= sum_j h_j V_j
__global__ void k_fvm_sub_combo(size_t n, int k, const double* __restrict__ V, const double* __restrict__ h,
                                double* __restrict__ w) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = w[i];
    for (int j = 0; j < k; ++j) s -= h[j] * V[(size_t)j * n + i];
    w[i] = s;
}
// y = sum_j c_j V_j
__global__ void k_fvm_combo(size_t n, int k, const double* __restrict__ V, const double* __restrict__ c,
                            double* __restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += c[j] * V[(size_t)j * n + i];
    y[i] = s;
}
// part[j][block] = partial sums of V_j . w over a fixed grid-stride split
__global__ void k_fvm_dots_partial(size_t n, const double* __restrict__ V, const double* __restrict__ w,
                                   double* __restrict__ part) {
    __shared__ double red[32];
    const int j = blockIdx.y;
    const double* v = V + (size_t)j * n;
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        s += v[i] * w[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[(size_t)j * gridDim.x + blockIdx.x] = s;
}
__global__ void k_fvm_dots_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double red[32];
    const int j = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[(size_t)j * nb + i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) out[j] = s;
}

int launched(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return BTE_OK;
    return fvm_fail(BTE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int fvm_alloc(bte_fvm* h, void** p, size_t bytes) {
    if (cudaMalloc(p, std::max<size_t>(bytes, 8)) != cudaSuccess) return fvm_fail(BTE_ERR_ALLOC, "device allocation failed");
    h->allocs.push_back(*p);
    return BTE_OK;
}

void fvm_free(bte_fvm* h) {
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
}

int sweep_rc(int rc, const char* what) {
    if (rc == 0) return BTE_OK;
    return fvm_fail(BTE_ERR_CUDA, std::string(what) + ": " + bte_sweep_last_error());
}

// Y = rhs_mvec(X) on stream s
int fvm_mvec(bte_fvm* h, const FvmCoef& c, const double* E, const double* X, double* Y, cudaStream_t s) {
    const FvmView v = view_of(h);
    const size_t nrx = (size_t)h->Nr * h->Nx;
    k_fvm_moment<<<fblocks(nrx), FT, 0, s>>>(v, X, h->M);
    if (int rc = launched("k_fvm_moment")) return rc;
    if (int rc = sweep_rc(bte_dgemm_nn(h->Nr, h->Nx, h->Nr, h->gain, h->Nr, h->M, h->Nx, h->T, h->Nx, s), "gain product"))
        return rc;
    k_fvm_mvec<<<fblocks(h->N), FT, 0, s>>>(v, c, E, h->T, X, Y);
    h->launches += 3;
    return launched("k_fvm_mvec");
}

// Y = the op-split step applied to X (aE = cE E must already be in h->aE, ax v_r in h->axvr)
int fvm_precond(bte_fvm* h, double hstep, const double* X, double* Y, cudaStream_t s) {
    const FvmView v = view_of(h);
    const int Nr = h->Nr, Nvt = h->Nvt, Nx = h->Nx;
    const size_t nrx = (size_t)Nr * Nx;
    k_fvm_moment<<<fblocks(nrx), FT, 0, s>>>(v, X, h->M);
    if (int rc = launched("k_fvm_moment")) return rc;
    if (int rc = sweep_rc(bte_dgemm_nn(Nr, Nx, Nr, h->H, Nr, h->M, Nx, h->T, Nx, s), "collision inverse")) return rc;
    const size_t xsm = ((size_t)XT_L * (Nx + 1) + 2 * (size_t)h->ndx * Nx) * sizeof(double);
    const size_t rsm = 2 * (size_t)h->ndr * Nr * sizeof(double), tsm = 2 * (size_t)h->ndt * Nvt * sizeof(double);
    if (h->ndr > SW_NDMAX || h->ndt > SW_NDMAX || h->ndx > SW_NDMAX || xsm > 200 * 1024 || rsm > 200 * 1024 ||
        tsm > 200 * 1024) {
        // stencils wider than the register recurrence or x lines longer than the staged rows:
        // the drop-in sweeps on permuted copies
        k_fvm_coll_permute<<<fblocks(h->N), FT, 0, s>>>(v, h->dinv, h->T, X, h->A);   // (Nx, Nvt, Nr)
        if (int rc = launched("k_fvm_coll_permute")) return rc;
        int rc = sweep_rc(bte_adv_be_sweep(0, h->vrL, h->vrR, h->aE, h->cos_t, hstep, h->A, h->Bf, h->ndr, Nr, Nvt, Nx, s),
                          "v_r sweep");
        if (!rc) rc = sweep_rc(bte_permute3(Nx, Nvt, Nr, 0, 2, 1, h->Bf, h->A, s), "layout");   // (Nx, Nr, Nvt)
        if (!rc)
            rc = sweep_rc(bte_adv_be_sweep(1, h->vtL, h->vtR, h->aE, h->vr, hstep, h->A, h->Bf, h->ndt, Nr, Nvt, Nx, s),
                          "v_theta sweep");
        if (!rc) rc = sweep_rc(bte_permute3(Nx, Nr, Nvt, 1, 2, 0, h->Bf, h->A, s), "layout");   // (Nr, Nvt, Nx)
        if (!rc) rc = sweep_rc(bte_fvm_inflow_zero(Nr, Nvt, Nx, h->vt, h->A, s), "inflow");
        if (!rc)
            rc = sweep_rc(bte_adv_be_sweep(2, h->xL, h->xR, h->axvr, h->cos_t, hstep, h->A, Y, h->ndx, Nr, Nvt, Nx, s),
                          "x sweep");
        h->launches += 10;
        return rc;
    }
    k_fvm_coll_apply<<<fblocks(h->N), FT, 0, s>>>(v, h->dinv, h->T, X, h->A);   // natural layout
    if (int rc = launched("k_fvm_coll_apply")) return rc;
    // the three sweeps in place on the natural layout, coalesced (no layout swaps)
    // the v_r lines are few (Nvt Nx) and long: small CTAs spread them over the SMs
    if (bte_raise_smem_limit((const void*)k_fvm_sweep_vr, rsm) != cudaSuccess ||
        bte_raise_smem_limit((const void*)k_fvm_sweep_vt, tsm) != cudaSuccess ||
        bte_raise_smem_limit((const void*)k_fvm_sweep_x, xsm) != cudaSuccess)
        return fvm_fail(BTE_ERR_ARG, "sweep lines too long for the shared-memory sweeps");
    // h->Bf (the drop-in path's scratch) holds the diagonal reciprocals of the v_r, then the x sweep
    k_fvm_diag_rcp<<<fblocks(h->N), FT, 0, s>>>(v, 0, h->aE, h->axvr, hstep, h->Bf);
    if (int rc = launched("k_fvm_diag_rcp")) return rc;
    k_fvm_sweep_vr<<<(unsigned)(((size_t)Nvt * Nx + 31) / 32), 32, rsm, s>>>(v, h->aE, hstep, h->A, h->Bf);
    if (int rc = launched("k_fvm_sweep_vr")) return rc;
    k_fvm_sweep_vt<<<fblocks((size_t)Nr * Nx), FT, tsm, s>>>(v, h->aE, hstep, h->A);
    if (int rc = launched("k_fvm_sweep_vt")) return rc;
    k_fvm_diag_rcp<<<fblocks(h->N), FT, 0, s>>>(v, 2, h->aE, h->axvr, hstep, h->Bf);
    if (int rc = launched("k_fvm_diag_rcp")) return rc;
    k_fvm_sweep_x<<<(unsigned)((Nr * Nvt + XT_L - 1) / XT_L), XT_T, xsm, s>>>(v, h->axvr, hstep, h->A, Y, h->Bf);
    h->launches += 8;
    return launched("k_fvm_sweep_x");
}

// aE = cE E on the device, axvr = ax v_r
int fvm_coefficients(bte_fvm* h, double cE, double ax, const double* E, cudaStream_t s) {
    k_fvm_scale<<<fblocks(h->Nx), FT, 0, s>>>((size_t)h->Nx, cE, E, h->aE);
    k_fvm_scale<<<fblocks(h->Nr), FT, 0, s>>>((size_t)h->Nr, ax, h->vr, h->axvr);
    h->launches += 2;
    return launched("coefficients");
}

FvmSl sl_of(const bte_fvm* h, const FvmCoef& c) {
    FvmSl sl;
    sl.Nr = h->Nr; sl.Nvt = h->Nvt; sl.Nx = h->Nx;
    sl.vr = h->vr; sl.vt = h->vt; sl.cos_t = h->cos_t; sl.vrp = h->vrp; sl.vta = h->vta; sl.x = h->xg;
    sl.vmin = h->sl_vmin;
    sl.cX = c.dt * c.ax;
    sl.cE = c.dt * c.tau * c.cA;
    return sl;
}

// Y = step_adv_vx_sl(V) (Y must not alias V)
int fvm_sl(bte_fvm* h, const FvmCoef& c, const double* E, const double* V, double* Y, cudaStream_t s) {
    k_fvm_sl<<<fblocks(h->N), FT, 0, s>>>(sl_of(h, c), E, V, Y);
    ++h->launches;
    return launched("k_fvm_sl");
}

// Y = (I - c C)^-1 B in the natural layout (Y must not alias B)
int fvm_coll_solve(bte_fvm* h, const double* B, double* Y, cudaStream_t s) {
    const FvmView v = view_of(h);
    const size_t nrx = (size_t)h->Nr * h->Nx;
    k_fvm_moment<<<fblocks(nrx), FT, 0, s>>>(v, B, h->M);
    if (int rc = launched("k_fvm_moment")) return rc;
    if (int rc = sweep_rc(bte_dgemm_nn(h->Nr, h->Nx, h->Nr, h->H, h->Nr, h->M, h->Nx, h->T, h->Nx, s), "collision inverse"))
        return rc;
    k_fvm_coll_apply<<<fblocks(h->N), FT, 0, s>>>(v, h->dinv, h->T, B, Y);
    h->launches += 3;
    return launched("k_fvm_coll_apply");
}

struct DeviceOps {
    bte_fvm* h;
    cudaStream_t s;
    FvmCoef c;
    const double* E;
    double hstep;
    size_t N;
    double *B, *X, *R, *W, *Z, *T, *Kr;
    bool identity;   // pc_type "none": no preconditioner

    int matvec(const double* x, double* y) { return fvm_mvec(h, c, E, x, y, s); }
    int precond(const double* x, double* y) {
        if (!identity) return fvm_precond(h, hstep, x, y, s);
        if (cudaMemcpyAsync(y, x, N * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return fvm_fail(BTE_ERR_CUDA, "copy failed");
        return BTE_OK;
    }
    int dots(int k, const double* V, const double* w, double* out) {
        k_fvm_dots_partial<<<dim3(FVM_RED, k), FT, 0, s>>>(N, V, w, h->part);
        k_fvm_dots_final<<<k, FT, 0, s>>>(FVM_RED, h->part, h->hd);
        h->launches += 2;
        if (int rc = launched("dots")) return rc;
        if (cudaMemcpyAsync(out, h->hd, (size_t)k * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return fvm_fail(BTE_ERR_CUDA, "dots: copy to the host failed");
        return BTE_OK;
    }
    int to_device(int k, const double* host) {
        if (cudaMemcpyAsync(h->hd, host, (size_t)k * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return fvm_fail(BTE_ERR_CUDA, "coefficient copy failed");
        return BTE_OK;
    }
    int sub_combo(int k, const double* V, const double* hh, double* w) {
        if (int rc = to_device(k, hh)) return rc;
        k_fvm_sub_combo<<<fblocks(N), FT, 0, s>>>(N, k, V, h->hd, w);
        ++h->launches;
        return launched("sub_combo");
    }
    int combo(int k, const double* V, const double* cc, double* y) {
        if (int rc = to_device(k, cc)) return rc;
        k_fvm_combo<<<fblocks(N), FT, 0, s>>>(N, k, V, h->hd, y);
        ++h->launches;
        return launched("combo");
    }
    int scale(double a, const double* x, double* y) {
        k_fvm_scale<<<fblocks(N), FT, 0, s>>>(N, a, x, y);
        ++h->launches;
        return launched("scale");
    }
    int axpy(double a, const double* x, double* y) {
        k_fvm_axpy<<<fblocks(N), FT, 0, s>>>(N, a, x, y);
        ++h->launches;
        return launched("axpy");
    }
    int sub(const double* a, const double* b, double* cc) {
        k_fvm_sub<<<fblocks(N), FT, 0, s>>>(N, a, b, cc);
        ++h->launches;
        return launched("sub");
    }
};

bool coef_ok(const bte_fvm_coef* c) {
    return c && std::isfinite(c->dt) && std::isfinite(c->dtx) && std::isfinite(c->tau) && std::isfinite(c->kappa) &&
           std::isfinite(c->cA) && std::isfinite(c->ax);
}

FvmCoef coef_of(const bte_fvm_coef* c) {
    FvmCoef f;
    f.dt = c->dt; f.dtx = c->dtx; f.tau = c->tau; f.kappa = c->kappa; f.cA = c->cA; f.ax = c->ax;
    return f;
}

}  // namespace

extern "C" {

const char* bte_fvm_last_error(void) { return g_fvm_err.c_str(); }

int bte_fvm_create(int device, int Nr, int Nvt, int Nx, int ndr, int ndt, int ndx, const double* vr, const double* vt,
                   const double* w, const double* loss, const double* gain, const double* vr_l2r,
                   const double* vr_r2l, const double* vt_l2r, const double* vt_r2l, const double* x_l2r,
                   const double* x_r2l, bte_fvm** out) {
    if (!out) return fvm_fail(BTE_ERR_ARG, "bte_fvm_create: null handle pointer");
    *out = nullptr;
    if (!vr || !vt || !w || !loss || !gain || !vr_l2r || !vr_r2l || !vt_l2r || !vt_r2l || !x_l2r || !x_r2l)
        return fvm_fail(BTE_ERR_ARG, "bte_fvm_create: null argument");
    if (Nr < 2 || Nvt < 2 || (Nvt & 1) || Nx < 2 || ndr < 1 || ndt < 1 || ndx < 1 || ndr > Nr || ndt > Nvt || ndx > Nx)
        return fvm_fail(BTE_ERR_ARG, "bte_fvm_create: sizes out of range (Nr, Nx >= 2, Nvt even >= 2, 1 <= nd <= N)");
    const size_t N = (size_t)Nr * Nvt * Nx;
    if (N > ((size_t)1 << 31)) return fvm_fail(BTE_ERR_ARG, "bte_fvm_create: Nr * Nvt * Nx above 2^31");
    for (int r = 0; r < Nr; ++r)
        if (!(vr[r] > 0.0)) return fvm_fail(BTE_ERR_ARG, "bte_fvm_create: cell centres must be positive");
    if (cudaSetDevice(device) != cudaSuccess) return fvm_fail(BTE_ERR_CUDA, "cudaSetDevice failed");
    bte_fvm* h = new bte_fvm();
    h->device = device; h->Nr = Nr; h->Nvt = Nvt; h->Nx = Nx; h->ndr = ndr; h->ndt = ndt; h->ndx = ndx; h->N = N;
    int rc = BTE_OK;
    auto A = [&](double** p, size_t count) { if (rc == BTE_OK) rc = fvm_alloc(h, (void**)p, count * 8); };
    A(&h->vr, Nr); A(&h->vt, Nvt); A(&h->cos_t, Nvt); A(&h->w, Nvt); A(&h->loss, Nr); A(&h->gain, (size_t)Nr * Nr);
    A(&h->vrL, (size_t)ndr * Nr); A(&h->vrR, (size_t)ndr * Nr); A(&h->vtL, (size_t)ndt * Nvt);
    A(&h->vtR, (size_t)ndt * Nvt); A(&h->xL, (size_t)ndx * Nx); A(&h->xR, (size_t)ndx * Nx);
    A(&h->dinv, Nr); A(&h->H, (size_t)Nr * Nr);
    A(&h->M, (size_t)Nr * Nx); A(&h->T, (size_t)Nr * Nx); A(&h->aE, Nx); A(&h->axvr, Nr);
    A(&h->A, N); A(&h->Bf, N); A(&h->B, N); A(&h->X, N); A(&h->R, N); A(&h->W, N); A(&h->Z, N); A(&h->Tv, N);
    if (rc == BTE_OK) rc = fvm_alloc(h, (void**)&h->north, Nvt);
    if (rc != BTE_OK) {
        fvm_free(h);
        delete h;
        return rc;
    }
    std::vector<double> cth(Nvt);
    std::vector<int8_t> north(Nvt);
    const double half_pi = 0.5 * 3.14159265358979323846;
    for (int j = 0; j < Nvt; ++j) {
        cth[j] = std::cos(vt[j]);
        north[j] = vt[j] <= half_pi ? 1 : 0;
    }
    struct Cp { void* d; const void* s; size_t b; };
    const Cp cps[] = {{h->vr, vr, (size_t)Nr * 8}, {h->vt, vt, (size_t)Nvt * 8}, {h->cos_t, cth.data(), (size_t)Nvt * 8},
                      {h->w, w, (size_t)Nvt * 8}, {h->loss, loss, (size_t)Nr * 8}, {h->gain, gain, (size_t)Nr * Nr * 8},
                      {h->vrL, vr_l2r, (size_t)ndr * Nr * 8}, {h->vrR, vr_r2l, (size_t)ndr * Nr * 8},
                      {h->vtL, vt_l2r, (size_t)ndt * Nvt * 8}, {h->vtR, vt_r2l, (size_t)ndt * Nvt * 8},
                      {h->xL, x_l2r, (size_t)ndx * Nx * 8}, {h->xR, x_r2l, (size_t)ndx * Nx * 8},
                      {h->north, north.data(), (size_t)Nvt}};
    for (const Cp& c : cps)
        if (cudaMemcpy(c.d, c.s, c.b, cudaMemcpyHostToDevice) != cudaSuccess) {
            fvm_free(h);
            delete h;
            return fvm_fail(BTE_ERR_CUDA, "bte_fvm_create: copy of the set-up failed");
        }
    *out = h;
    return BTE_OK;
}

int bte_fvm_destroy(bte_fvm* h) {
    if (!h) return BTE_OK;
    cudaSetDevice(h->device);
    cudaFree(h->Kr);   // the GMRES buffers, sized by the largest restart so far
    cudaFree(h->part);
    cudaFree(h->hd);
    fvm_free(h);
    delete h;
    return BTE_OK;
}

long long bte_fvm_launches(const bte_fvm* h) { return h ? h->launches : 0; }

int bte_fvm_set_collision_inverse(bte_fvm* h, const double* dinv, const double* H) {
    if (!h || !dinv || !H) return fvm_fail(BTE_ERR_ARG, "bte_fvm_set_collision_inverse: null argument");
    cudaSetDevice(h->device);
    if (cudaMemcpy(h->dinv, dinv, (size_t)h->Nr * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->H, H, (size_t)h->Nr * h->Nr * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return fvm_fail(BTE_ERR_CUDA, "bte_fvm_set_collision_inverse: copy failed");
    h->have_inverse = true;
    return BTE_OK;
}

int bte_fvm_mvec(bte_fvm* h, const bte_fvm_coef* c, const double* E, const double* X, double* Y, void* stream) {
    if (!h || !E || !X || !Y) return fvm_fail(BTE_ERR_ARG, "bte_fvm_mvec: null argument");
    if (!coef_ok(c)) return fvm_fail(BTE_ERR_ARG, "bte_fvm_mvec: coefficients missing or not finite");
    if (X == Y) return fvm_fail(BTE_ERR_ARG, "bte_fvm_mvec: Y must not alias X");
    cudaSetDevice(h->device);
    return fvm_mvec(h, coef_of(c), E, X, Y, (cudaStream_t)stream);
}

int bte_fvm_precond(bte_fvm* h, double cE, double ax, double hstep, const double* E, const double* X, double* Y,
                    void* stream) {
    if (!h || !E || !X || !Y) return fvm_fail(BTE_ERR_ARG, "bte_fvm_precond: null argument");
    if (!h->have_inverse) return fvm_fail(BTE_ERR_STATE, "bte_fvm_precond: no collision inverse set");
    if (X == Y || X == h->A || X == h->Bf) return fvm_fail(BTE_ERR_ARG, "bte_fvm_precond: Y must not alias X");
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = fvm_coefficients(h, cE, ax, E, s)) return rc;
    return fvm_precond(h, hstep, X, Y, s);
}

int bte_fvm_set_sl_grid(bte_fvm* h, const double* x, double vmin, double vmax) {
    if (!h || !x) return fvm_fail(BTE_ERR_ARG, "bte_fvm_set_sl_grid: null argument");
    const int Nr = h->Nr, Nvt = h->Nvt, Nx = h->Nx;
    std::vector<double> hv(Nvt);
    if (cudaSetDevice(h->device) != cudaSuccess ||
        cudaMemcpy(hv.data(), h->vt, (size_t)Nvt * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fvm_fail(BTE_ERR_CUDA, "bte_fvm_set_sl_grid: copy failed");
    std::vector<double> hr(Nr);
    if (cudaMemcpy(hr.data(), h->vr, (size_t)Nr * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fvm_fail(BTE_ERR_CUDA, "bte_fvm_set_sl_grid: copy failed");
    const double pi = 3.14159265358979323846;
    std::vector<double> vrp(Nr + 2), vta(Nvt + 2);
    vrp[0] = vmin;
    vrp[Nr + 1] = vmax;
    for (int r = 0; r < Nr; ++r) vrp[r + 1] = hr[r];
    vta[0] = 0.0;
    vta[Nvt + 1] = pi;
    for (int j = 0; j < Nvt; ++j) vta[j + 1] = hv[Nvt - 1 - j];
    bool ascending = true;
    for (int i = 0; i + 1 < Nr + 2; ++i) ascending = ascending && vrp[i] < vrp[i + 1];
    for (int i = 0; i + 1 < Nvt + 2; ++i) ascending = ascending && vta[i] < vta[i + 1];
    for (int i = 0; i + 1 < Nx; ++i) ascending = ascending && x[i] < x[i + 1];
    if (!ascending)
        return fvm_fail(BTE_ERR_ARG, "bte_fvm_set_sl_grid: need vmin < vr < vmax, ordinates in (0, pi) descending, x ascending");
    int rc = BTE_OK;
    if (!h->have_sl) {
        if (rc == BTE_OK) rc = fvm_alloc(h, (void**)&h->xg, (size_t)Nx * 8);
        if (rc == BTE_OK) rc = fvm_alloc(h, (void**)&h->vrp, (size_t)(Nr + 2) * 8);
        if (rc == BTE_OK) rc = fvm_alloc(h, (void**)&h->vta, (size_t)(Nvt + 2) * 8);
        if (rc != BTE_OK) return rc;
    }
    if (cudaMemcpy(h->xg, x, (size_t)Nx * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->vrp, vrp.data(), (size_t)(Nr + 2) * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->vta, vta.data(), (size_t)(Nvt + 2) * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return fvm_fail(BTE_ERR_CUDA, "bte_fvm_set_sl_grid: copy failed");
    h->sl_vmin = vmin;
    h->have_sl = true;
    return BTE_OK;
}

int bte_fvm_sl_advect(bte_fvm* h, const bte_fvm_coef* c, const double* E, const double* V, double* Y, void* stream) {
    if (!h || !E || !V || !Y) return fvm_fail(BTE_ERR_ARG, "bte_fvm_sl_advect: null argument");
    if (!coef_ok(c)) return fvm_fail(BTE_ERR_ARG, "bte_fvm_sl_advect: coefficients missing or not finite");
    if (!h->have_sl) return fvm_fail(BTE_ERR_STATE, "bte_fvm_sl_advect: no semi-Lagrangian grid set");
    if (V == Y) return fvm_fail(BTE_ERR_ARG, "bte_fvm_sl_advect: Y must not alias V");
    cudaSetDevice(h->device);
    return fvm_sl(h, coef_of(c), E, V, Y, (cudaStream_t)stream);
}

int bte_fvm_sl_step(bte_fvm* h, const bte_fvm_coef* c, const double* E, const double* V, double* Y, void* stream) {
    if (!h || !E || !V || !Y) return fvm_fail(BTE_ERR_ARG, "bte_fvm_sl_step: null argument");
    if (!coef_ok(c)) return fvm_fail(BTE_ERR_ARG, "bte_fvm_sl_step: coefficients missing or not finite");
    if (!h->have_sl) return fvm_fail(BTE_ERR_STATE, "bte_fvm_sl_step: no semi-Lagrangian grid set");
    if (!h->have_inverse) return fvm_fail(BTE_ERR_STATE, "bte_fvm_sl_step: no collision inverse set");
    if (V == Y || V == h->A || Y == h->A) return fvm_fail(BTE_ERR_ARG, "bte_fvm_sl_step: Y must not alias V");
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = fvm_sl(h, coef_of(c), E, V, h->A, s)) return rc;
    return fvm_coll_solve(h, h->A, Y, s);
}

int bte_fvm_step(bte_fvm* h, const bte_fvm_coef* c, double alpha, int pc_mode, const double* E, double* V, double rtol,
                 double atol, int restart, int max_iter, double* info4, void* stream) {
    if (!h || !E || !V || !info4) return fvm_fail(BTE_ERR_ARG, "bte_fvm_step: null argument");
    if (!coef_ok(c) || !std::isfinite(alpha)) return fvm_fail(BTE_ERR_ARG, "bte_fvm_step: coefficients not finite");
    if (restart < 1 || restart > 500 || max_iter < 0) return fvm_fail(BTE_ERR_ARG, "bte_fvm_step: 1 <= restart <= 500");
    if (pc_mode < 0 || pc_mode > 2) return fvm_fail(BTE_ERR_ARG, "bte_fvm_step: pc_mode must be 0, 1 or 2");
    if (pc_mode != 2 && !h->have_inverse) return fvm_fail(BTE_ERR_STATE, "bte_fvm_step: no collision inverse set");
    cudaSetDevice(h->device);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t N = h->N;
    if (restart > h->kcap) {
        double *Kr = nullptr, *part = nullptr, *hd = nullptr;
        if (cudaMalloc((void**)&Kr, (size_t)(restart + 1) * N * 8) != cudaSuccess)
            return fvm_fail(BTE_ERR_ALLOC, "bte_fvm_step: Krylov basis allocation failed");
        if (cudaMalloc((void**)&part, (size_t)(restart + 1) * FVM_RED * 8) != cudaSuccess ||
            cudaMalloc((void**)&hd, (size_t)(restart + 1) * 8) != cudaSuccess) {
            cudaFree(Kr);
            cudaFree(part);
            return fvm_fail(BTE_ERR_ALLOC, "bte_fvm_step: reduction buffers allocation failed");
        }
        if (h->Kr) {
            cudaFree(h->Kr);
            cudaFree(h->part);
            cudaFree(h->hd);
        }
        h->Kr = Kr;
        h->part = part;
        h->hd = hd;
        h->kcap = restart;
    }
    const FvmCoef fc = coef_of(c);
    if (int rc = fvm_coefficients(h, fc.tau * fc.cA, fc.ax, E, s)) return rc;
    // right-hand side: V with its inflow values zeroed (bte_1d3v_solver.py:1907-1911)
    if (cudaMemcpyAsync(h->B, V, N * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return fvm_fail(BTE_ERR_CUDA, "bte_fvm_step: copy of the state failed");
    if (int rc = sweep_rc(bte_fvm_inflow_zero(h->Nr, h->Nvt, h->Nx, h->vt, h->B, s), "inflow")) return rc;
    DeviceOps op{h, s, fc, E, alpha * fc.dt, N, h->B, h->X, h->R, h->W, h->Z, h->Tv, h->Kr, pc_mode == 2};
    FvmGmresInfo info{};
    if (int rc = pc_mode == 1 ? fvm_gmres_left(op, restart, rtol, atol, max_iter, &info)
                              : fvm_gmres(op, restart, rtol, atol, max_iter, &info))
        return rc;
    if (cudaMemcpyAsync(V, h->X, N * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fvm_fail(BTE_ERR_CUDA, "bte_fvm_step: copy of the solution failed");
    info4[0] = info.iterations;
    info4[1] = info.rnorm;
    info4[2] = info.bnorm > 0.0 ? info.rnorm / info.bnorm : 0.0;
    info4[3] = info.converged ? 0.0 : 1.0;
    return BTE_OK;
}

}  // extern "C"
