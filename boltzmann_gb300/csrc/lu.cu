// Batched dense LU with partial pivoting and triangular solves (FP64 / FP32).
//
// Replaces the explicit batched inverse of the Newton Jacobian
// (xp.linalg.inv in bte_0d3v_batched.py:856-880, applied at :933-934): the solver only
// needs J^-1 r, so the library factors once and substitutes.
//
// Storage: each matrix is ROW-major, A[r * ld + c], rows 0..N-1, columns 0..NC-1 (NC = N,
// or N + 1 when the right-hand side is appended as column N and eliminated with the
// matrix). Rows are never exchanged in memory: the factorization returns perm, and the
// row of L\U at pivot position r lives in the original row perm[r] (partial pivoting
// picks the first index of max |a|, as LAPACK's i?amax).
//
// Two kernels, one CTA per matrix:
//   k_lu_left   (N <= 512)  left-looking by 32-column blocks. A block lives in registers
//               (thread = 4 columns x N/32 rows) while the previous L panels stream through
//               shared memory read-only; its 32 x 32 U blocks are solved in shared memory;
//               then the block's panel is factored in shared memory (two barriers per
//               column) and written once. No read-modify-write of a trailing matrix.
//   k_lu_right  (any N)     right-looking by panels (trailing matrix in global memory),
//               for the largest systems.
// (k_lu_tc in lu_tc.cu is the FP32 tensor-core kernel; k_lus_* below split one FP64
// factorization over many CTAs.)
#include <cstdint>
#include <algorithm>
#include "bte_common.cuh"

namespace {

constexpr int LU_THREADS = 256;
constexpr int LU_MAX_N = LU_THREADS * 8;

// |v| with the sign bit cleared: -0.0 must give +0.0, because the FP32 pivot search compares
// the bit patterns of |v| (a -0.0 kept its sign bit and outranked every positive value)
__device__ inline float tabs(float v) { return fabsf(v); }
__device__ inline double tabs(double v) { return fabs(v); }

template <typename T> struct LuOcc { static constexpr int value = 1; };
template <> struct LuOcc<float> { static constexpr int value = 2; };

__host__ __device__ inline size_t align16(size_t bytes) { return (bytes + 15) & ~(size_t)15; }

// 4 / 8 consecutive elements from 16-byte aligned shared memory
__device__ inline void ld4(const float* p, float v[4]) {
    float4 a = *reinterpret_cast<const float4*>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ inline void ld4(const double* p, double v[4]) {
    double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
template <typename T>
__device__ inline void ld8(const T* p, T v[8]) {
    ld4(p, v);
    ld4(p + 4, v + 4);
}

// asynchronous global -> shared copies of one element (Ampere+ cp.async; no alignment
// requirement beyond the element size)
__device__ inline void cp_async_elem(float* smem, const float* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ inline void cp_async_elem(double* smem, const double* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NG>
__device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NG) : "memory"); }

// Unblocked partial-pivoting factorization of a panel in shared memory, column-major
// P[c * ldp + r], rows 0..mrows-1 (pivot positions base..base+mrows-1), pivots on the
// first kbr columns, interchanges and updates on ncol columns. Thread t owns rows
// t, t + nt, ... (at most ROWS), so each column costs two barriers: after the warp
// candidates and after the interchange. perm (shared, position -> stored row) and
// inf (first zero pivot, 1-based, thread 0) are updated.
// Pivot candidate of a warp: the largest |a| (first row on ties) among the lanes'
// candidates. FP32 uses the integer max-reduction instruction on the bit pattern of
// |a| (monotone for non-negative floats; NaN never wins) and a ballot for the lane;
// FP64 compares through shuffles.
__device__ inline void warp_argmax(float& best, int& bi) {
    unsigned key = (best >= 0.0f) ? __float_as_uint(best) : 0u;
    unsigned kmax = __reduce_max_sync(0xffffffffu, key);
    unsigned ball = __ballot_sync(0xffffffffu, key == kmax);
    // among the lanes holding the max, the smallest row index
    int cand = (key == kmax) ? bi : 0x7fffffff;
    int rmin = (int)__reduce_min_sync(0xffffffffu, (unsigned)cand);
    (void)ball;
    best = __uint_as_float(kmax);
    bi = rmin;
}
__device__ inline void warp_argmax(double& best, int& bi) {
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
}
__device__ inline float recip(float d) { return __frcp_rn(d); }
__device__ inline double recip(double d) { return 1.0 / d; }

// Unblocked partial-pivoting factorization of a panel in shared memory, column-major
// P[c * ldp + r], rows 0..mrows-1 (pivot positions base..base+mrows-1), pivots on the
// first kbr columns, interchanges and updates on ncol <= 32 columns. Thread t owns rows
// t, t + nt, ... (at most ROWS), so each column costs two barriers: after the warp
// candidates and after the interchange. perm (shared, position -> stored row) and
// inf (first zero pivot, 1-based, thread 0) are updated.
template <typename T, int ROWS, int NBMAX>
__device__ void panel_factor(T* P, int ldp, int mrows, int kbr, int ncol, int* perm, int base, int& inf,
                             T* redv, int* redi) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int j = 0; j < kbr; ++j) {
        T best = T(-1);
        int bi = mrows;
#pragma unroll
        for (int k = 0; k < ROWS; ++k) {
            int r = tid + k * nt;
            if (r >= j && r < mrows) {
                T v = tabs(P[j * ldp + r]);
                if (v > best) { best = v; bi = r; }
            }
        }
        warp_argmax(best, bi);
        if ((tid & 31) == 0) { redv[tid >> 5] = best; redi[tid >> 5] = bi; }
        __syncthreads();
        T b = redv[0];
        int pr = redi[0];
#pragma unroll
        for (int w = 1; w < LU_THREADS / 32; ++w) {
            T vb = redv[w];
            int ib = redi[w];
            if (vb > b || (vb == b && ib < pr)) { b = vb; pr = ib; }
        }
        if (pr >= mrows || !(b >= T(0))) pr = j;  // no valid candidate (NaN): keep the diagonal
        if (tid < 32) {
            if (pr != j && tid < ncol) {
                T t0 = P[tid * ldp + j];
                P[tid * ldp + j] = P[tid * ldp + pr];
                P[tid * ldp + pr] = t0;
            }
            if (tid == 0) {
                if (pr != j) {
                    int t1 = perm[base + j];
                    perm[base + j] = perm[base + pr];
                    perm[base + pr] = t1;
                }
                if (!(b != T(0)) && inf == 0) inf = base + j + 1;
            }
        }
        __syncthreads();
        const T d = P[j * ldp + j];
        const T inv = (d != T(0)) ? recip(d) : T(0);
#pragma unroll
        for (int k = 0; k < ROWS; ++k) {
            int r = tid + k * nt;
            if (r > j && r < mrows) {
                T l = P[j * ldp + r] * inv;
                P[j * ldp + r] = l;
                for (int c = j + 1; c < ncol; ++c) P[c * ldp + r] -= l * P[c * ldp + j];
            }
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------------
// left-looking kernel, N <= 32 * RPT
// ---------------------------------------------------------------------------------
constexpr int LB = 32;          // block width
constexpr int LDL = LB + 1;     // padded row of a staged L panel
constexpr int LDU = LB + 4;     // padded row of a U block (16-byte aligned rows)

__host__ __device__ inline int left_ldp(int N) { return (N % 2 == 0) ? N + 1 : N; }
// two staging buffers for the streamed L panels (the panel factorization reuses the first)
__host__ __device__ inline size_t left_stage_elems(int N) {
    size_t stage = (size_t)N * LDL;
    size_t panel = (size_t)left_ldp(N) * LB;
    return (stage > panel ? stage : panel);
}
__host__ __device__ inline size_t left_smem_bytes(int N, size_t w) {
    return align16((size_t)N * 4) + align16((size_t)LB * LDU * w) + 2 * align16(left_stage_elems(N) * w);
}

template <typename T, int RPT>
__global__ void __launch_bounds__(LU_THREADS, LuOcc<T>::value)
k_lu_left(int N, int NC, T* __restrict__ A, int ld, long long stride, int32_t* __restrict__ perm_out,
          int32_t* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char smraw[];
    int* perm = reinterpret_cast<int*>(smraw);
    T* Ub = reinterpret_cast<T*>(smraw + align16((size_t)N * 4));
    T* Ls0 = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(Ub) + align16((size_t)LB * LDU * sizeof(T)));
    T* Ls1 = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(Ls0) + align16(left_stage_elems(N) * sizeof(T)));
    __shared__ T redv[LU_THREADS / 32];
    __shared__ int redi[LU_THREADS / 32];
    const int mat = blockIdx.x;
    T* a = A + (size_t)mat * stride;
    const int tid = threadIdx.x, rg = tid >> 3, cg = tid & 7;
    const int w = tid >> 5, lane = tid & 31;
    const int ldp = left_ldp(N);
    for (int r = tid; r < N; r += LU_THREADS) perm[r] = r;
    int inf = 0;
    __syncthreads();
    const int nblk = (NC + LB - 1) / LB;
    for (int jb = 0; jb < nblk; ++jb) {
        const int c0 = jb * LB;
        T acc[RPT][4];
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = rg + 32 * i;
            const T* row = a + (size_t)(r < N ? perm[r] : 0) * ld;
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                const int c = c0 + cg * 4 + cc;
                acc[i][cc] = (r < N && c < NC) ? row[c] : T(0);
            }
        }
        // ---- left-looking updates with the previous panels; panel kb + 1 streams into the
        //      other staging buffer (cp.async) while panel kb is used
        auto stage = [&](int kb, T* buf) {
            const int k0 = kb * LB;
            for (int r = k0 + w; r < N; r += LU_THREADS / 32)
                cp_async_elem(buf + r * LDL + lane, a + (size_t)perm[r] * ld + k0 + lane);
            cp_async_commit();
        };
        if (jb > 0) stage(0, Ls0);
        for (int kb = 0; kb < jb; ++kb) {
            const int k0 = kb * LB;
            T* Ls = (kb & 1) ? Ls1 : Ls0;
            if (kb + 1 < jb) {
                stage(kb + 1, (kb & 1) ? Ls0 : Ls1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            // rows k0..k0+31 of the block are final: U_kj = L_kk^-1 (those rows)
#pragma unroll
            for (int i = 0; i < RPT; ++i)
                if (i == kb)
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) Ub[rg * LDU + cg * 4 + cc] = acc[i][cc];
            __syncthreads();
            if (tid < LB) {
                T x[LB];
#pragma unroll
                for (int j = 0; j < LB; ++j) x[j] = Ub[j * LDU + tid];
#pragma unroll
                for (int j = 1; j < LB; ++j) {
                    T s = x[j];
#pragma unroll
                    for (int i = 0; i < j; ++i) s -= Ls[(k0 + j) * LDL + i] * x[i];
                    x[j] = s;
                }
#pragma unroll
                for (int j = 0; j < LB; ++j) Ub[j * LDU + tid] = x[j];
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < RPT; ++i)
                if (i == kb) ld4(Ub + rg * LDU + cg * 4, acc[i]);
            // rows below: acc -= L[r][k0..k0+31] U_kj
#pragma unroll 4
            for (int kk = 0; kk < LB; ++kk) {
                T u[4];
                ld4(Ub + kk * LDU + cg * 4, u);
#pragma unroll
                for (int i = 0; i < RPT; ++i) {
                    const int r = rg + 32 * i;
                    if (i > kb && r < N) {
                        const T l = Ls[r * LDL + kk];
#pragma unroll
                        for (int cc = 0; cc < 4; ++cc) acc[i][cc] -= l * u[cc];
                    }
                }
            }
            __syncthreads();  // this buffer and Ub are reused two panels / one panel later
        }
        // ---- rows above the panel are final (U): write them now, freeing the registers
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = rg + 32 * i;
            if (r < c0 && r < N) {
                T* row = a + (size_t)perm[r] * ld;
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) {
                    const int c = c0 + cg * 4 + cc;
                    if (c < NC) row[c] = acc[i][cc];
                }
            }
        }
        // ---- factor the block's panel (positions c0..N-1) in shared memory
        const int mrows = N - c0;
        const int kbr = min(LB, N - c0);
        const int ncol = min(LB, NC - c0);
        T* Pn = Ls0;
        if (mrows > 0) {
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int r = rg + 32 * i;
                if (r >= c0 && r < N)
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) Pn[(cg * 4 + cc) * ldp + (r - c0)] = acc[i][cc];
            }
            __syncthreads();
            panel_factor<T, 2, LB>(Pn, ldp, mrows, kbr, ncol, perm, c0, inf, redv, redi);
        }
        // ---- write the panel rows of the block from shared memory
        for (int e = tid; e < mrows * LB; e += LU_THREADS) {
            const int rr = e / LB, c = e % LB;
            if (c < ncol) a[(size_t)perm[c0 + rr] * ld + c0 + c] = Pn[c * ldp + rr];
        }
        __syncthreads();
    }
    for (int r = tid; r < N; r += LU_THREADS) perm_out[(size_t)mat * N + r] = perm[r];
    if (tid == 0) info[mat] = inf;
}

// ---------------------------------------------------------------------------------
// right-looking kernel (any N <= LU_MAX_N), same storage convention
// ---------------------------------------------------------------------------------
__host__ __device__ inline int lu_ldp(int N) { return ((N + 7) & ~7) + 9; }
__host__ __device__ inline int lu_ldu(int NC) { return ((NC + 7) & ~7) + 8; }
__host__ __device__ inline size_t lu_smem_bytes(int N, int NC, int NB, size_t w) {
    return align16((size_t)N * 4) + align16((size_t)lu_ldp(N) * NB * w) + (size_t)NB * lu_ldu(NC) * w;
}

template <typename T, int NB, int ROWS>
__global__ void __launch_bounds__(LU_THREADS, LuOcc<T>::value)
k_lu_right(int N, int NC, T* __restrict__ A, int ld, long long stride, int32_t* __restrict__ perm_out,
           int32_t* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char smraw[];
    int* perm = reinterpret_cast<int*>(smraw);
    T* P = reinterpret_cast<T*>(smraw + align16((size_t)N * 4));
    const int ldp = lu_ldp(N), ldu = lu_ldu(NC);
    T* U = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(P) + align16((size_t)ldp * NB * sizeof(T)));
    __shared__ T redv[LU_THREADS / 32];
    __shared__ int redi[LU_THREADS / 32];
    const int mat = blockIdx.x;
    T* a = A + (size_t)mat * stride;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int r = tid; r < N; r += nt) perm[r] = r;
    int inf = 0;
    __syncthreads();
    for (int k0 = 0; k0 < N; k0 += NB) {
        const int kb = min(NB, N - k0);
        const int mrows = N - k0;
        for (int e = tid; e < mrows * NB; e += nt) {
            int r = e / NB, c = e % NB;
            P[c * ldp + r] = (c < kb) ? a[(size_t)perm[k0 + r] * ld + k0 + c] : T(0);
        }
        __syncthreads();
        panel_factor<T, ROWS, NB>(P, ldp, mrows, kb, kb, perm, k0, inf, redv, redi);
        for (int e = tid; e < mrows * kb; e += nt) {
            int r = e / kb, c = e % kb;
            a[(size_t)perm[k0 + r] * ld + k0 + c] = P[c * ldp + r];
        }
        const int c0g = k0 + kb;
        const int ncol = NC - c0g;
        if (ncol <= 0) break;
        // U12 = L11^-1 A12 (unit lower), thread per column
        for (int c = tid; c < ncol; c += nt) {
            T x[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) x[j] = (j < kb) ? a[(size_t)perm[k0 + j] * ld + c0g + c] : T(0);
#pragma unroll
            for (int j = 0; j < NB; ++j) {
#pragma unroll
                for (int i = 0; i < j; ++i) x[j] -= P[i * ldp + j] * x[i];
            }
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                U[j * ldu + c] = x[j];
                if (j < kb) a[(size_t)perm[k0 + j] * ld + c0g + c] = x[j];
            }
        }
        for (int e = tid; e < NB * 8; e += nt) U[(e / 8) * ldu + ncol + e % 8] = T(0);
        __syncthreads();
        // A22 -= L21 U12, 8 x 8 register tiles
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
                    T* row = a + (size_t)perm[k0 + r] * ld + c0g + cc0;
#pragma unroll
                    for (int jx = 0; jx < 8; ++jx)
                        if (cc0 + jx < ncol) row[jx] -= acc[i][jx];
                }
            }
        }
        __syncthreads();
    }
    for (int r = tid; r < N; r += nt) perm_out[(size_t)mat * N + r] = perm[r];
    if (tid == 0) info[mat] = inf;
}

// ---------------------------------------------------------------------------------
// split right-looking kernel (kernel 6, FP64): one factorization spread over many CTAs.
// Per panel of NB columns, three launches in stream order:
//   k_lus_panel   one CTA per matrix: partial pivoting of the panel in shared memory
//                 (perm updated in global memory; rows are never exchanged), panel written back;
//   k_lus_trsm    one CTA per (matrix, 64 columns right of the panel): U12 = L11^-1 A12;
//   k_lus_update  one CTA per (matrix, 64 x 64 tile of the trailing matrix): A22 -= L21 U12
//                 from shared-memory copies of the L21 and U12 tiles, 4 x 4 register tiles.
// The one-CTA-per-matrix kernels run each matrix on one SM. GB300 issues about 2 DFMA per
// clock per SM, so a lone FP64 factorization of N = 385 takes milliseconds there and one of
// N = 1281 a fifth of a second: what the few points of an FP64 lane pay per Newton
// iteration. Split, the trailing updates of even one matrix spread over the GPU and the
// serial part is the panels' pivot searches. Same arithmetic for a matrix whatever P is.
// ---------------------------------------------------------------------------------
constexpr int SP_T = 64;          // trailing tile edge
constexpr int SP_LDS = SP_T + 1;  // padded shared-memory row of a tile

__host__ __device__ inline int split_ldp(int mrows) { return mrows | 1; }
__host__ __device__ inline size_t split_panel_smem(int mrows, int NB, size_t w) {
    return align16((size_t)mrows * 4) + (size_t)split_ldp(mrows) * NB * w;
}

template <typename T, int NB, int ROWS>
__global__ void __launch_bounds__(LU_THREADS)
k_lus_panel(int N, int k0, T* __restrict__ A, int ld, long long stride, int32_t* __restrict__ perm_g,
            int32_t* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int mrows = N - k0, kb = min(NB, mrows), ldp = split_ldp(mrows);
    int* ps = reinterpret_cast<int*>(smraw);
    T* P = reinterpret_cast<T*>(smraw + align16((size_t)mrows * 4));
    __shared__ T redv[LU_THREADS / 32];
    __shared__ int redi[LU_THREADS / 32];
    const int mat = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    T* a = A + (size_t)mat * stride;
    int32_t* pg = perm_g + (size_t)mat * N;
    for (int r = tid; r < mrows; r += nt) ps[r] = (k0 == 0) ? r : pg[k0 + r];
    __syncthreads();
    for (int e = tid; e < mrows * kb; e += nt) {
        const int r = e / kb, c = e % kb;
        P[c * ldp + r] = a[(size_t)ps[r] * ld + k0 + c];
    }
    __syncthreads();
    int inf = 0;
    panel_factor<T, ROWS, NB>(P, ldp, mrows, kb, kb, ps, 0, inf, redv, redi);
    for (int e = tid; e < mrows * kb; e += nt) {
        const int r = e / kb, c = e % kb;
        a[(size_t)ps[r] * ld + k0 + c] = P[c * ldp + r];
    }
    for (int r = tid; r < mrows; r += nt) pg[k0 + r] = ps[r];
    if (tid == 0) {
        int cur = (k0 == 0) ? 0 : info[mat];
        if (cur == 0 && inf != 0) cur = k0 + inf;
        info[mat] = cur;
    }
}

template <typename T, int NB>
__global__ void __launch_bounds__(SP_T)
k_lus_trsm(int N, int NC, int k0, int ncb, T* __restrict__ A, int ld, long long stride,
           const int32_t* __restrict__ perm_g) {
    __shared__ T L[NB][NB + 1];
    __shared__ int pr[NB];
    const int kb = min(NB, N - k0), c0g = k0 + kb;
    const int mat = blockIdx.x / ncb, cb = blockIdx.x % ncb;
    T* a = A + (size_t)mat * stride;
    const int32_t* pg = perm_g + (size_t)mat * N;
    const int tid = threadIdx.x;
    if (tid < NB) pr[tid] = (tid < kb) ? pg[k0 + tid] : 0;
    __syncthreads();
    for (int e = tid; e < NB * NB; e += SP_T) {
        const int i = e / NB, j = e % NB;
        L[i][j] = (i < kb && j < kb) ? a[(size_t)pr[i] * ld + k0 + j] : T(0);
    }
    __syncthreads();
    const int c = c0g + cb * SP_T + tid;
    if (c >= NC) return;
    T x[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) x[j] = (j < kb) ? a[(size_t)pr[j] * ld + c] : T(0);
#pragma unroll
    for (int j = 1; j < NB; ++j) {
#pragma unroll
        for (int i = 0; i < j; ++i) x[j] -= L[j][i] * x[i];
    }
#pragma unroll
    for (int j = 0; j < NB; ++j)
        if (j < kb) a[(size_t)pr[j] * ld + c] = x[j];
}

template <typename T, int NB>
__global__ void __launch_bounds__(256)
k_lus_update(int N, int NC, int k0, int nrb, int ncb, T* __restrict__ A, int ld, long long stride,
             const int32_t* __restrict__ perm_g) {
    __shared__ T Ls[NB][SP_LDS];  // L21 tile, transposed: Ls[k][r]
    __shared__ T Us[NB][SP_LDS];  // U12 tile: Us[k][c]
    __shared__ int prow[SP_T];
    __shared__ int pk[NB];
    const int kb = min(NB, N - k0), c0g = k0 + kb;
    const int mr = N - c0g, ncol = NC - c0g;
    const int per = nrb * ncb;
    const int mat = blockIdx.x / per, t = blockIdx.x % per, rb = t / ncb, cb = t % ncb;
    T* a = A + (size_t)mat * stride;
    const int32_t* pg = perm_g + (size_t)mat * N;
    const int tid = threadIdx.x;
    if (tid < SP_T) {
        const int r = rb * SP_T + tid;
        prow[tid] = (r < mr) ? pg[c0g + r] : -1;
    }
    if (tid < NB) pk[tid] = (tid < kb) ? pg[k0 + tid] : 0;
    __syncthreads();
    for (int e = tid; e < SP_T * NB; e += 256) {
        const int r = e / NB, k = e % NB;
        Ls[k][r] = (prow[r] >= 0 && k < kb) ? a[(size_t)prow[r] * ld + k0 + k] : T(0);
    }
    for (int e = tid; e < NB * SP_T; e += 256) {
        const int k = e / SP_T, c = e % SP_T;
        const int cl = cb * SP_T + c;
        Us[k][c] = (k < kb && cl < ncol) ? a[(size_t)pk[k] * ld + c0g + cl] : T(0);
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll 8
    for (int k = 0; k < NB; ++k) {
        T av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = Ls[k][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = Us[k][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] += av[i] * bv[j];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int pr = prow[ty + 16 * i];
        if (pr < 0) continue;
        T* row = a + (size_t)pr * ld + c0g + cb * SP_T;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = tx + 16 * j;
            if (cb * SP_T + c < ncol) row[c] -= acc[i][j];
        }
    }
}

template <typename T, int NB, int ROWS>
cudaError_t launch_split_panel(int P, int N, int k0, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                               cudaStream_t s) {
    const size_t sm = split_panel_smem(N - k0, NB, sizeof(T));
    cudaError_t e = bte_raise_smem_limit((const void*)k_lus_panel<T, NB, ROWS>, sm);
    if (e != cudaSuccess) return e;
    k_lus_panel<T, NB, ROWS><<<P, LU_THREADS, sm, s>>>(N, k0, A, ld, stride, piv, info);
    return cudaGetLastError();
}

template <typename T, int NB>
cudaError_t factor_split_nb(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s) {
    for (int k0 = 0; k0 < N; k0 += NB) {
        const int mrows = N - k0, kb = std::min(NB, mrows);
        cudaError_t e;
        if (mrows <= LU_THREADS) e = launch_split_panel<T, NB, 1>(P, N, k0, A, ld, stride, piv, info, s);
        else if (mrows <= 2 * LU_THREADS) e = launch_split_panel<T, NB, 2>(P, N, k0, A, ld, stride, piv, info, s);
        else if (mrows <= 4 * LU_THREADS) e = launch_split_panel<T, NB, 4>(P, N, k0, A, ld, stride, piv, info, s);
        else e = launch_split_panel<T, NB, 8>(P, N, k0, A, ld, stride, piv, info, s);
        if (e != cudaSuccess) return e;
        const int c0g = k0 + kb, ncol = NC - c0g, mr = N - c0g;
        if (ncol <= 0) break;
        const int ncb = (ncol + SP_T - 1) / SP_T;
        k_lus_trsm<T, NB><<<(unsigned)P * ncb, SP_T, 0, s>>>(N, NC, k0, ncb, A, ld, stride, piv);
        if (mr > 0) {
            const int nrb = (mr + SP_T - 1) / SP_T;
            k_lus_update<T, NB><<<(unsigned)P * nrb * ncb, 256, 0, s>>>(N, NC, k0, nrb, ncb, A, ld, stride, piv);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// panel width: as wide as the panel's shared memory allows (<= 200 KB)
template <typename T>
cudaError_t factor_split(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                         cudaStream_t s) {
    if (split_panel_smem(N, 32, sizeof(T)) <= 200 * 1024)
        return factor_split_nb<T, 32>(P, N, NC, A, ld, stride, piv, info, s);
    if (split_panel_smem(N, 16, sizeof(T)) <= 200 * 1024)
        return factor_split_nb<T, 16>(P, N, NC, A, ld, stride, piv, info, s);
    return factor_split_nb<T, 8>(P, N, NC, A, ld, stride, piv, info, s);
}

// Substitution for one right-hand side per matrix. mode 0: full solve (gather b by perm,
// unit-lower forward, upper backward); mode 1: backward only (the RHS was eliminated as
// column N during the factorization). Rows of position r are read from stored row perm[r].
// With a list, CTA i solves with matrix mats[i] and right-hand side i.
template <typename T>
__global__ void __launch_bounds__(LU_THREADS)
k_lu_solve(int N, const T* __restrict__ A, int ld, long long stride, const int32_t* __restrict__ perm,
           T* __restrict__ b, int mode, const int32_t* __restrict__ mats) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* x = reinterpret_cast<T*>(smraw);
    const int mat = mats ? mats[blockIdx.x] : (int)blockIdx.x;
    const T* a = A + (size_t)mat * stride;
    const int32_t* pm = perm + (size_t)mat * N;
    T* bb = b + (size_t)blockIdx.x * N;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    if (mode == 1) {
        for (int i = tid; i < N; i += nt) x[i] = a[(size_t)pm[i] * ld + N];
        __syncthreads();
    } else {
        for (int i = tid; i < N; i += nt) x[i] = bb[pm[i]];
        __syncthreads();
        for (int r0 = 0; r0 < N; r0 += 32) {
            const int rb = min(32, N - r0);
            for (int i = wid; i < rb; i += nw) {
                const T* row = a + (size_t)pm[r0 + i] * ld;
                T s = T(0);
                for (int c = lane; c < r0; c += 32) s += row[c] * x[c];
                s = warp_sum(s);
                if (lane == 0) x[r0 + i] -= s;
            }
            __syncthreads();
            if (wid == 0) {
                T xi = (lane < rb) ? x[r0 + lane] : T(0);
                const T* rowl = a + (size_t)pm[r0 + min(lane, rb - 1)] * ld;
                for (int j = 0; j < rb; ++j) {
                    T xj = __shfl_sync(0xffffffffu, xi, j);
                    if (lane > j && lane < rb) xi -= rowl[r0 + j] * xj;
                }
                if (lane < rb) x[r0 + lane] = xi;
            }
            __syncthreads();
        }
    }
    for (int r1 = N; r1 > 0; r1 -= 32) {
        const int r0 = max(0, r1 - 32), rb = r1 - r0;
        for (int i = wid; i < rb; i += nw) {
            const T* row = a + (size_t)pm[r0 + i] * ld;
            T s = T(0);
            for (int c = r1 + lane; c < N; c += 32) s += row[c] * x[c];
            s = warp_sum(s);
            if (lane == 0) x[r0 + i] -= s;
        }
        __syncthreads();
        if (wid == 0) {
            T xi = (lane < rb) ? x[r0 + lane] : T(0);
            const T* rowl = a + (size_t)pm[r0 + min(lane, rb - 1)] * ld;
            for (int j = rb - 1; j >= 0; --j) {
                T d = a[(size_t)pm[r0 + j] * ld + r0 + j];
                T xj = __shfl_sync(0xffffffffu, xi, j);
                xj = (d != T(0)) ? xj / d : xj;
                if (lane == j) xi = xj;
                if (lane < j) xi -= rowl[r0 + j] * xj;
            }
            if (lane < rb) x[r0 + lane] = xi;
        }
        __syncthreads();
    }
    for (int i = tid; i < N; i += nt) bb[i] = x[i];
}

template <typename T, int RPT>
cudaError_t launch_left(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                        cudaStream_t s) {
    size_t sm = left_smem_bytes(N, sizeof(T));
    cudaError_t e = bte_raise_smem_limit((const void*)k_lu_left<T, RPT>, sm);
    if (e != cudaSuccess) return e;
    k_lu_left<T, RPT><<<P, LU_THREADS, sm, s>>>(N, NC, A, ld, stride, piv, info);
    return cudaGetLastError();
}

template <typename T, int NB, int ROWS>
cudaError_t launch_right_r(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                           cudaStream_t s) {
    size_t sm = lu_smem_bytes(N, NC, NB, sizeof(T));
    cudaError_t e = bte_raise_smem_limit((const void*)k_lu_right<T, NB, ROWS>, sm);
    if (e != cudaSuccess) return e;
    k_lu_right<T, NB, ROWS><<<P, LU_THREADS, sm, s>>>(N, NC, A, ld, stride, piv, info);
    return cudaGetLastError();
}

template <typename T, int NB>
cudaError_t launch_right(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                         cudaStream_t s) {
    if (N <= 2 * LU_THREADS) return launch_right_r<T, NB, 2>(P, N, NC, A, ld, stride, piv, info, s);
    if (N <= 4 * LU_THREADS) return launch_right_r<T, NB, 4>(P, N, NC, A, ld, stride, piv, info, s);
    return launch_right_r<T, NB, 8>(P, N, NC, A, ld, stride, piv, info, s);
}

// panel width of the right-looking kernel: as wide as fits in shared memory (<= 200 KB)
template <typename T>
int pick_nb(int N, int NC) {
    for (int nb : {32, 16, 8})
        if (lu_smem_bytes(N, NC, nb, sizeof(T)) <= 200 * 1024) return nb;
    return 0;
}

template <typename T>
cudaError_t factor_right(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                         cudaStream_t s) {
    int nb = pick_nb<T>(N, NC);
    if (nb == 32) return launch_right<T, 32>(P, N, NC, A, ld, stride, piv, info, s);
    if (nb == 16) return launch_right<T, 16>(P, N, NC, A, ld, stride, piv, info, s);
    if (nb == 8) return launch_right<T, 8>(P, N, NC, A, ld, stride, piv, info, s);
    return cudaErrorInvalidValue;
}

}  // namespace

int bte_lu_tc_max_n();
cudaError_t bte_lu_factor_tc(int P, int N, int NC, float* A, int ld, long long stride, int32_t* piv, int32_t* info,
                             cudaStream_t s, int variant);

// Factor P matrices in place; piv[P][N] receives perm (position -> stored row).
// kernel: 0 = automatic (FP32, N <= 512: tensor cores; FP32 above: right-looking; FP64:
// right-looking), 1 = right-looking, 2 = FP32 with the trailing updates on the tensor cores
// (lu_tc.cu; N <= 512; 256 threads, two CTAs per SM), 3 = left-looking SIMT (N <= 512), 4 = as
// 2 with one CTA per SM, 5 = as 2 with 128 threads per CTA, 6 = FP64 split over many CTAs per
// matrix (panel, triangular solve and 64 x 64 trailing tiles as separate launches).
template <typename T>
cudaError_t bte_lu_factor_t(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s, int kernel) {
    if (P <= 0) return cudaSuccess;
    if (N < 1 || N > LU_MAX_N || NC < N || NC > N + 1 || ld < NC) return cudaErrorInvalidValue;
    // FP64: the right-looking kernel (the left-looking one serialises FP64 substitutions)
    if (sizeof(T) == 8 && kernel == 0) kernel = 1;
    if (kernel == 6) {
        if constexpr (sizeof(T) == 8) {
            return factor_split<T>(P, N, NC, A, ld, stride, piv, info, s);
        } else {
            return cudaErrorInvalidValue;
        }
    }
    if (kernel == 2 || kernel == 4 || kernel == 5) {
        if (sizeof(T) != 4 || N > bte_lu_tc_max_n()) return cudaErrorInvalidValue;
        return bte_lu_factor_tc(P, N, NC, reinterpret_cast<float*>(A), ld, stride, piv, info, s,
                                kernel == 2 ? 0 : (kernel == 4 ? 1 : 2));
    }
    if (kernel == 3) {
        if (N > 512) return cudaErrorInvalidValue;
    } else if (kernel == 0 && sizeof(T) == 4 && N <= bte_lu_tc_max_n()) {
        // FP32 default: the tensor-core kernel, faster than the left-looking SIMT kernel at
        // every measured size from N = 33 to 512 (4096 matrices: 1.1x at N = 33 and 385,
        // 1.3x at N = 129 and 257, 1.7x at N = 512)
        return bte_lu_factor_tc(P, N, NC, reinterpret_cast<float*>(A), ld, stride, piv, info, s, 0);
    }
    if (kernel == 3) kernel = 0;
    if (kernel == 0 && N <= 128) return launch_left<T, 4>(P, N, NC, A, ld, stride, piv, info, s);
    if (kernel == 0 && N <= 256) return launch_left<T, 8>(P, N, NC, A, ld, stride, piv, info, s);
    if (kernel == 0 && N <= 384) return launch_left<T, 12>(P, N, NC, A, ld, stride, piv, info, s);
    if (kernel == 0 && N <= 416) return launch_left<T, 13>(P, N, NC, A, ld, stride, piv, info, s);
    if (kernel == 0 && N <= 512) return launch_left<T, 16>(P, N, NC, A, ld, stride, piv, info, s);
    return factor_right<T>(P, N, NC, A, ld, stride, piv, info, s);
}

template <typename T>
cudaError_t bte_lu_solve_t(int P, int N, const T* A, int ld, long long stride, const int32_t* piv, T* b, int mode,
                           cudaStream_t s, const int32_t* mats) {
    if (P <= 0) return cudaSuccess;
    size_t sm = (size_t)N * sizeof(T);
    cudaError_t e = bte_raise_smem_limit((const void*)k_lu_solve<T>, sm);
    if (e != cudaSuccess) return e;
    k_lu_solve<T><<<P, LU_THREADS, sm, s>>>(N, A, ld, stride, piv, b, mode, mats);
    return cudaGetLastError();
}

template cudaError_t bte_lu_factor_t<double>(int, int, int, double*, int, long long, int32_t*, int32_t*, cudaStream_t, int);
template cudaError_t bte_lu_factor_t<float>(int, int, int, float*, int, long long, int32_t*, int32_t*, cudaStream_t, int);
template cudaError_t bte_lu_solve_t<double>(int, int, const double*, int, long long, const int32_t*, double*, int,
                                            cudaStream_t, const int32_t*);
template cudaError_t bte_lu_solve_t<float>(int, int, const float*, int, long long, const int32_t*, float*, int,
                                           cudaStream_t, const int32_t*);
