// Batched dense LU with partial pivoting and triangular solves (FP64 / FP32).
//
// Replaces the explicit batched inverse of the Newton Jacobian
// (xp.linalg.inv in bte_0d3v_batched.py:856-880, applied at :933-934): the solver only
// needs J^-1 r, so the library factors once and substitutes.
//
// Layout: each matrix is ROW-major, A[r * ld + c], rows 0..N-1, columns 0..NC-1 (NC = N, or
// N + 1 when the right-hand side is appended as column N and eliminated with the matrix).
// One CTA factors one matrix, right-looking and blocked by NB columns:
//   panel (rows k0.., cols k0..k0+NB) staged in shared memory and factored there
//   (pivot = first index of max |a|, as LAPACK's i?amax); the panel's row interchanges
//   are applied to every other column (LAPACK convention, so L is stored in final row
//   order); U12 = L11^-1 A12 by column-parallel substitution; A22 -= L21 U12 by a
//   register-tiled (8 x 8 per thread) product read from shared memory.
#include <cstdint>
#include <algorithm>
#include "bte_common.cuh"

namespace {

constexpr int LU_THREADS = 256;
constexpr int LU_MAX_N = LU_THREADS * 8;  // panel rows per thread (ROWS) are 2, 4 or 8

template <typename T> __device__ inline T tabs(T v) { return v < T(0) ? -v : v; }

__host__ __device__ inline int lu_ldp(int N) { return ((N + 7) & ~7) + 9; }
__host__ __device__ inline int lu_ldu(int NC) { return ((NC + 7) & ~7) + 8; }
__host__ __device__ inline size_t lu_smem_elems(int N, int NC, int NB) {
    // U must start 16-byte aligned: round the panel part up to a multiple of 8 elements
    return (((size_t)lu_ldp(N) * NB + 7) & ~(size_t)7) + (size_t)NB * lu_ldu(NC);
}

// 8 consecutive elements from 16-byte aligned shared memory
__device__ inline void ld8(const float* p, float v[8]) {
    float4 a = *reinterpret_cast<const float4*>(p), b = *reinterpret_cast<const float4*>(p + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ inline void ld8(const double* p, double v[8]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double2 a = *reinterpret_cast<const double2*>(p + 2 * i);
        v[2 * i] = a.x; v[2 * i + 1] = a.y;
    }
}

// FP32: two CTAs per SM (the panel factorization of one overlaps the other's update);
// FP64: one, the FP64 pipe is the bound and the register tile needs the room
template <typename T> struct LuOcc { static constexpr int value = 1; };
template <> struct LuOcc<float> { static constexpr int value = 2; };

template <typename T, int NB, int LU_ROWS>
__global__ void __launch_bounds__(LU_THREADS, LuOcc<T>::value)
k_lu_factor(int N, int NC, T* __restrict__ A, int ld, long long stride, int32_t* __restrict__ piv,
            int32_t* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* sm = reinterpret_cast<T*>(smraw);
    const int mat = blockIdx.x;
    T* a = A + (size_t)mat * stride;
    int32_t* pv = piv + (size_t)mat * N;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int ldp = lu_ldp(N);              // panel rows (column-major in smem), odd: no bank conflicts
    const int ldu = lu_ldu(NC);             // U12 row length, multiple of 8 plus 8 of padding
    T* P = sm;                                            // ldp x NB
    T* U = sm + (((size_t)ldp * NB + 7) & ~(size_t)7);    // NB x ldu
    __shared__ T redv[LU_THREADS / 32];
    __shared__ int redi[LU_THREADS / 32];
    int inf = 0;

    for (int k0 = 0; k0 < N; k0 += NB) {
        const int kb = min(NB, N - k0);
        const int mrows = N - k0;
        // ---- load panel: rows k0..N-1, columns k0..k0+kb-1
        for (int e = tid; e < mrows * NB; e += nt) {
            int r = e / NB, c = e % NB;
            P[c * ldp + r] = (c < kb) ? a[(size_t)(k0 + r) * ld + k0 + c] : T(0);
        }
        __syncthreads();
        // ---- unblocked factorization of the panel. Thread t owns panel rows t, t + nt, ...
        // (at most LU_ROWS of them), so the pivot search reads only its own rows and each
        // column costs two barriers: after the warp candidates, after the row interchange.
        for (int j = 0; j < kb; ++j) {
            T best = T(-1);
            int bi = mrows;  // sentinel: larger than any row
#pragma unroll
            for (int k = 0; k < LU_ROWS; ++k) {
                int r = tid + k * nt;
                if (r >= j && r < mrows) {
                    T v = tabs(P[j * ldp + r]);
                    if (v > best || (v == best && r < bi)) { best = v; bi = r; }
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                T ov = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if ((tid & 31) == 0) { redv[tid >> 5] = best; redi[tid >> 5] = bi; }
            __syncthreads();
            T b = redv[0];
            int pr = redi[0];
            for (int w = 1; w < nt / 32; ++w)
                if (redv[w] > b || (redv[w] == b && redi[w] < pr)) { b = redv[w]; pr = redi[w]; }
            if (pr >= mrows) pr = j;  // all candidates NaN: keep the diagonal
            if (tid < 32) {
                if (pr != j && tid < kb) {
                    T t0 = P[tid * ldp + j];
                    P[tid * ldp + j] = P[tid * ldp + pr];
                    P[tid * ldp + pr] = t0;
                }
                if (tid == 0) {
                    pv[k0 + j] = k0 + pr;
                    if (!(b != T(0)) && inf == 0) inf = k0 + j + 1;
                }
            }
            __syncthreads();
            const T d = P[j * ldp + j];
            const T inv = (d != T(0)) ? T(1) / d : T(0);
#pragma unroll
            for (int k = 0; k < LU_ROWS; ++k) {
                int r = tid + k * nt;
                if (r > j && r < mrows) {
                    T l = P[j * ldp + r] * inv;
                    P[j * ldp + r] = l;
                    for (int c = j + 1; c < kb; ++c) P[c * ldp + r] -= l * P[c * ldp + j];
                }
            }
        }
        __syncthreads();
        // ---- write the panel back
        for (int e = tid; e < mrows * kb; e += nt) {
            int r = e / kb, c = e % kb;
            a[(size_t)(k0 + r) * ld + k0 + c] = P[c * ldp + r];
        }
        // ---- row interchanges on the columns outside the panel (coalesced: thread per column)
        for (int c = tid; c < NC; c += nt) {
            if (c >= k0 && c < k0 + kb) continue;
            for (int j = 0; j < kb; ++j) {
                int prow = pv[k0 + j];
                if (prow != k0 + j) {
                    T t0 = a[(size_t)(k0 + j) * ld + c];
                    a[(size_t)(k0 + j) * ld + c] = a[(size_t)prow * ld + c];
                    a[(size_t)prow * ld + c] = t0;
                }
            }
        }
        __syncthreads();
        const int c0g = k0 + kb;
        const int ncol = NC - c0g;
        if (ncol <= 0) break;
        // ---- U12 = L11^-1 A12 (unit lower), thread per column
        for (int c = tid; c < ncol; c += nt) {
            T x[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) x[j] = (j < kb) ? a[(size_t)(k0 + j) * ld + c0g + c] : T(0);
#pragma unroll
            for (int j = 0; j < NB; ++j) {
#pragma unroll
                for (int i = 0; i < j; ++i) x[j] -= P[i * ldp + j] * x[i];
            }
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                U[j * ldu + c] = x[j];
                if (j < kb) a[(size_t)(k0 + j) * ld + c0g + c] = x[j];
            }
        }
        for (int e = tid; e < NB * 8; e += nt) {  // zero the 8 columns past the end (tile overhang)
            int j = e / 8, c = ncol + e % 8;
            U[j * ldu + c] = T(0);
        }
        __syncthreads();
        // ---- A22 -= L21 U12, 8 x 8 register tiles, lanes along columns for coalescing
        const int mr = mrows - kb;
        if (mr > 0) {
            const int ntc = (ncol + 7) / 8, ntr = (mr + 7) / 8;
            for (int tile = tid; tile < ntr * ntc; tile += nt) {
                const int tc = tile % ntc, tr = tile / ntc;
                const int r0 = kb + tr * 8, cc0 = tc * 8;
                T acc[8][8];
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int jx = 0; jx < 8; ++jx) acc[i][jx] = T(0);
#pragma unroll 4
                for (int j = 0; j < kb; ++j) {
                    T av[8], bv[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) av[i] = P[j * ldp + r0 + i];
                    ld8(U + j * ldu + cc0, bv);
#pragma unroll
                    for (int i = 0; i < 8; ++i)
#pragma unroll
                        for (int jx = 0; jx < 8; ++jx) acc[i][jx] += av[i] * bv[jx];
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    int r = r0 + i;
                    if (r >= mrows) break;
                    T* row = a + (size_t)(k0 + r) * ld + c0g + cc0;
#pragma unroll
                    for (int jx = 0; jx < 8; ++jx)
                        if (cc0 + jx < ncol) row[jx] -= acc[i][jx];
                }
            }
        }
        __syncthreads();
    }
    if (tid == 0) info[mat] = inf;
}

// Substitution for one right-hand side per matrix. mode 0: full solve (apply the
// interchanges, unit-lower forward, upper backward); mode 1: backward only (the RHS
// was eliminated as column N during the factorization and is read from there).
template <typename T>
__global__ void __launch_bounds__(LU_THREADS)
k_lu_solve(int N, const T* __restrict__ A, int ld, long long stride, const int32_t* __restrict__ piv,
           T* __restrict__ b, int mode) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* x = reinterpret_cast<T*>(smraw);
    const int mat = blockIdx.x;
    const T* a = A + (size_t)mat * stride;
    T* bb = b + (size_t)mat * N;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    if (mode == 1) {
        for (int i = tid; i < N; i += nt) x[i] = a[(size_t)i * ld + N];
        __syncthreads();
    } else {
        for (int i = tid; i < N; i += nt) x[i] = bb[i];
        __syncthreads();
        if (tid == 0) {
            const int32_t* pv = piv + (size_t)mat * N;
            for (int k = 0; k < N; ++k) {
                int p = pv[k];
                if (p != k) { T t0 = x[k]; x[k] = x[p]; x[p] = t0; }
            }
        }
        __syncthreads();
        // forward, unit lower, blocks of 32 rows
        for (int r0 = 0; r0 < N; r0 += 32) {
            const int rb = min(32, N - r0);
            // rows r0..r0+rb-1 minus contributions of solved x[0..r0)
            for (int i = wid; i < rb; i += nw) {
                const T* row = a + (size_t)(r0 + i) * ld;
                T s = T(0);
                for (int c = lane; c < r0; c += 32) s += row[c] * x[c];
                s = warp_sum(s);
                if (lane == 0) x[r0 + i] -= s;
            }
            __syncthreads();
            if (wid == 0) {
                T xi = (lane < rb) ? x[r0 + lane] : T(0);
                for (int j = 0; j < rb; ++j) {
                    T xj = __shfl_sync(0xffffffffu, xi, j);
                    if (lane > j && lane < rb) xi -= a[(size_t)(r0 + lane) * ld + r0 + j] * xj;
                }
                if (lane < rb) x[r0 + lane] = xi;
            }
            __syncthreads();
        }
    }
    // backward, upper, blocks of 32 rows from the bottom
    for (int r1 = N; r1 > 0; r1 -= 32) {
        const int r0 = max(0, r1 - 32), rb = r1 - r0;
        for (int i = wid; i < rb; i += nw) {
            const T* row = a + (size_t)(r0 + i) * ld;
            T s = T(0);
            for (int c = r1 + lane; c < N; c += 32) s += row[c] * x[c];
            s = warp_sum(s);
            if (lane == 0) x[r0 + i] -= s;
        }
        __syncthreads();
        if (wid == 0) {
            T xi = (lane < rb) ? x[r0 + lane] : T(0);
            for (int j = rb - 1; j >= 0; --j) {
                T d = a[(size_t)(r0 + j) * ld + r0 + j];
                T xj = __shfl_sync(0xffffffffu, xi, j);
                xj = (d != T(0)) ? xj / d : xj;
                if (lane == j) xi = xj;
                if (lane < j) xi -= a[(size_t)(r0 + lane) * ld + r0 + j] * xj;
            }
            if (lane < rb) x[r0 + lane] = xi;
        }
        __syncthreads();
    }
    for (int i = tid; i < N; i += nt) bb[i] = x[i];
}

template <typename T, int NB, int ROWS>
cudaError_t launch_factor_r(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s) {
    size_t sm = lu_smem_elems(N, NC, NB) * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(k_lu_factor<T, NB, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_lu_factor<T, NB, ROWS><<<P, LU_THREADS, sm, s>>>(N, NC, A, ld, stride, piv, info);
    return cudaGetLastError();
}

template <typename T, int NB>
cudaError_t launch_factor(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                          cudaStream_t s) {
    if (N <= 2 * LU_THREADS) return launch_factor_r<T, NB, 2>(P, N, NC, A, ld, stride, piv, info, s);
    if (N <= 4 * LU_THREADS) return launch_factor_r<T, NB, 4>(P, N, NC, A, ld, stride, piv, info, s);
    return launch_factor_r<T, NB, 8>(P, N, NC, A, ld, stride, piv, info, s);
}

}  // namespace

// panel width: as wide as fits in shared memory (<= 200 KB) to cut trailing-matrix passes
template <typename T>
static int pick_nb(int N, int NC) {
    const size_t cap = 200 * 1024;
    for (int nb : {32, 16, 8}) {
        size_t sm = lu_smem_elems(N, NC, nb) * sizeof(T);
        if (sm <= cap) return nb;
    }
    return 0;
}

template <typename T>
cudaError_t bte_lu_factor_t(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s) {
    if (P <= 0) return cudaSuccess;
    if (N > LU_MAX_N) return cudaErrorInvalidValue;  // panel rows per thread are bounded
    int nb = pick_nb<T>(N, NC);
    if (nb == 32) return launch_factor<T, 32>(P, N, NC, A, ld, stride, piv, info, s);
    if (nb == 16) return launch_factor<T, 16>(P, N, NC, A, ld, stride, piv, info, s);
    if (nb == 8) return launch_factor<T, 8>(P, N, NC, A, ld, stride, piv, info, s);
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t bte_lu_solve_t(int P, int N, const T* A, int ld, long long stride, const int32_t* piv, T* b, int mode,
                           cudaStream_t s) {
    if (P <= 0) return cudaSuccess;
    size_t sm = (size_t)N * sizeof(T);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_lu_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    k_lu_solve<T><<<P, LU_THREADS, sm, s>>>(N, A, ld, stride, piv, b, mode);
    return cudaGetLastError();
}

template cudaError_t bte_lu_factor_t<double>(int, int, int, double*, int, long long, int32_t*, int32_t*, cudaStream_t);
template cudaError_t bte_lu_factor_t<float>(int, int, int, float*, int, long long, int32_t*, int32_t*, cudaStream_t);
template cudaError_t bte_lu_solve_t<double>(int, int, const double*, int, long long, const int32_t*, double*, int, cudaStream_t);
template cudaError_t bte_lu_solve_t<float>(int, int, const float*, int, long long, const int32_t*, float*, int, cudaStream_t);
