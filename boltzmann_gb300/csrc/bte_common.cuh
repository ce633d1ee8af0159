// Shared device helpers for the batched 0D3V velocity-space library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include <map>
#include <mutex>
#include <utility>

#define BTE_SP_ORDER 3          // cubic B-splines only (the reference's driver default)
#define BTE_BAND 3              // |p - k| <= 3 for overlapping cubic supports
#define BTE_NB (2 * BTE_BAND + 1)

// Physical constants (CODATA 2018, identical doubles to scipy.constants 1.18).
#define BTE_QE 1.602176634e-19
#define BTE_ME 9.1093837139e-31
#define BTE_KB 1.380649e-23
#define BTE_EPS0 8.8541878188e-12
#define BTE_PI 3.141592653589793

// Error codes returned by every entry point (0 = success).
#define BTE_OK 0
#define BTE_ERR_ARG -1
#define BTE_ERR_CUDA -2
#define BTE_ERR_ALLOC -3
#define BTE_ERR_STATE -4

// Raise a kernel's dynamic shared-memory limit on the current device to at least `bytes`;
// it is never lowered. The limit starts at 48 KB minus the kernel's static shared memory
// (queried once per kernel and device), so a request below 48 KB can need it too. The limit
// belongs to the kernel, not to the calling thread: serving engines launch the same kernels
// from several host threads for grids of different sizes, and a smaller limit set by one of
// them between another's set and launch made that launch fail.
inline cudaError_t bte_raise_smem_limit(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> cur;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(kernel, dev);
    auto it = cur.find(key);
    if (it == cur.end()) {
        cudaFuncAttributes fa;
        if ((e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return e;
        it = cur.emplace(key, (size_t)fa.maxDynamicSharedSizeBytes).first;
    }
    if (bytes <= it->second) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) it->second = bytes;
    return e;
}

// Status codes written per point by the solver.
#define BTE_ST_CONVERGED 0      // ||r|| <= atol + rtol * ||r0||
#define BTE_ST_ROUNDOFF 1       // residual stopped decreasing at round-off level
#define BTE_ST_MAXITER 2        // iteration budget exhausted
#define BTE_ST_LINESEARCH 3     // step length fell below alpha_min
#define BTE_ST_NONFINITE 4      // residual or Jacobian became NaN / Inf
#define BTE_ST_SINGULAR 5       // zero pivot in the Jacobian factorization
#define BTE_ST_NEED_FP64 6      // internal: the mixed form hands the point to the FP64 path

// ----------------------------------------------------------------------------------
// Cubic B-spline evaluation: values and first/second derivatives of the 4 nonzero
// basis functions at x. Semantics of the reference (basis.py:387,411-412): each basis
// function is the clamped B-spline of the global knot vector restricted to its own
// support, 0 outside [t_0, t_n) (nan_to_num of scipy's extrapolate=False); at the right
// end x = t_n every basis element of the reference evaluates to 0, so the domain is
// half-open here too.
// The algorithm is the standard triangular recurrence for B-spline values and
// derivatives (Piegl & Tiller, "The NURBS Book", A2.2/A2.3), written here for degree 3.
// Returns the span index i (nonzero functions are i-3 .. i) or -1 outside the domain.
// ----------------------------------------------------------------------------------
__host__ __device__ inline int bspline_span(const double* t, int nsp, double x) {
    const int k = BTE_SP_ORDER;
    if (!(x >= t[k]) || !(x < t[nsp])) return -1;
    int lo = k, hi = nsp;  // t[lo] <= x < t[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (x >= t[mid]) lo = mid; else hi = mid;
    }
    return lo;
}

// ders[d][j] = d-th derivative of basis function (span-3+j) at x, d = 0..nd (nd <= 2).
__host__ __device__ inline int bspline_eval(const double* t, int nsp, double x, int nd, double ders[3][4]) {
    const int k = BTE_SP_ORDER;
    for (int d = 0; d < 3; ++d)
        for (int j = 0; j < 4; ++j) ders[d][j] = 0.0;
    int i = bspline_span(t, nsp, x);
    if (i < 0) return -1;
    double ndu[4][4], left[4], right[4];
    ndu[0][0] = 1.0;
    for (int j = 1; j <= k; ++j) {
        left[j] = x - t[i + 1 - j];
        right[j] = t[i + j] - x;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            ndu[j][r] = right[r + 1] + left[j - r];
            double tmp = ndu[r][j - 1] / ndu[j][r];
            ndu[r][j] = saved + right[r + 1] * tmp;
            saved = left[j - r] * tmp;
        }
        ndu[j][j] = saved;
    }
    for (int j = 0; j <= k; ++j) ders[0][j] = ndu[j][k];
    if (nd > 0) {
        double a[2][4];
        for (int r = 0; r <= k; ++r) {
            int s1 = 0, s2 = 1;
            a[0][0] = 1.0;
            for (int kk = 1; kk <= nd; ++kk) {
                double d = 0.0;
                int rk = r - kk, pk = k - kk;
                if (r >= kk) {
                    a[s2][0] = a[s1][0] / ndu[pk + 1][rk];
                    d = a[s2][0] * ndu[rk][pk];
                }
                int j1 = (rk >= -1) ? 1 : -rk;
                int j2 = (r - 1 <= pk) ? kk - 1 : k - r;
                for (int j = j1; j <= j2; ++j) {
                    a[s2][j] = (a[s1][j] - a[s1][j - 1]) / ndu[pk + 1][rk + j];
                    d += a[s2][j] * ndu[rk + j][pk];
                }
                if (r <= pk) {
                    a[s2][kk] = -a[s1][kk - 1] / ndu[pk + 1][r];
                    d += a[s2][kk] * ndu[r][pk];
                }
                ders[kk][r] = d;
                int tmp = s1; s1 = s2; s2 = tmp;
            }
        }
        double fac = (double)k;
        for (int kk = 1; kk <= nd; ++kk) {
            for (int j = 0; j <= k; ++j) ders[kk][j] *= fac;
            fac *= (double)(k - kk);
        }
    }
    return i;
}

// Value (derivative order d) of basis function p at x; 0 outside its support.
__host__ __device__ inline double bspline_basis(const double* t, int nsp, int p, double x, int d) {
    double ders[3][4];
    int i = bspline_eval(t, nsp, x, d, ders);
    if (i < 0) return 0.0;
    int j = p - (i - BTE_SP_ORDER);
    if (j < 0 || j > BTE_SP_ORDER) return 0.0;
    return ders[d][j];
}

// Linear interpolation of a tabulated cross section with end clamping, as
// scipy.interpolate.interp1d(kind="linear", bounds_error=False, fill_value=(y0, yN))
// does in collisions.py:79.
__host__ __device__ inline double interp_clamped(const double* xs, const double* ys, int n, double x) {
    if (x < xs[0]) return ys[0];
    if (x > xs[n - 1]) return ys[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (xs[mid] <= x) lo = mid; else hi = mid;
    }
    // scipy finds hi = searchsorted(xs, x, side='left') clipped to [1, n-1]
    int ihi = lo + 1;
    if (xs[lo] == x && lo > 0) { ihi = lo; lo = lo - 1; }
    double x0 = xs[lo], x1 = xs[ihi], y0 = ys[lo], y1 = ys[ihi];
    double slope = (y1 - y0) / (x1 - x0);
    return slope * (x - x0) + y0;
}

template <typename T>
__device__ inline T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ inline T block_sum(T v, T* red) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    T r = (threadIdx.x < nw) ? red[threadIdx.x] : T(0);
    if (wid == 0) r = warp_sum(r);
    if (threadIdx.x == 0) red[0] = r;
    __syncthreads();
    r = red[0];
    __syncthreads();
    return r;
}
