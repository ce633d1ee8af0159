// Batched banded kernels of the 1D3V finite-volume path: bidiagonal and banded triangular
// solves and products, the upwind backward-Euler sweeps along v_r, v_theta and x, and the
// block-sparse (BSR) unit upper triangular solve. Counterparts of the reference's CuPy raw
// kernels (BESolver/python/rawkernel.py:5-375) and of its BSR triangular solve
// (BESolver/cuda/spsm_bsr_upper_tri_solve.cu, BESolver/python/cusparse_spsolve.py), with
// the same layouts so that they are drop-ins.
//
// Layout: system-major, each system's N values contiguous (the reference's (bsz, N)
// arrays). Each system is a sequential recurrence, so one thread owns one system; its row
// stays in L1 (a 128-byte line serves 16 consecutive steps), so the DRAM traffic is the
// arrays once. Operators shared by all systems (the sweep's band matrices) are read through
// the read-only path.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "bte_common.cuh"

namespace {

constexpr int SW_THREADS = 128;
inline unsigned sw_blocks(long long n) { return (unsigned)((n + SW_THREADS - 1) / SW_THREADS); }

// lower: out[0] = b[0] / d[0], out[i] = (b[i] - s[i-1] out[i-1]) / d[i]   (rawkernel.py:5-19)
// upper: out[N-1] = b[N-1] / d[N-1], out[i] = (b[i] - s[i] out[i+1]) / d[i]   (:20-33)
__global__ void k_bidiag(int bsz, int N, const double* __restrict__ d, const double* __restrict__ sd,
                         const double* __restrict__ b, double* __restrict__ out, int lower) {
    const long long sys = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= bsz) return;
    const double* dd = d + sys * N;
    const double* ss = sd + sys * (N - 1);
    const double* bb = b + sys * N;
    double* o = out + sys * N;
    if (lower) {
        double x = bb[0] / dd[0];
        o[0] = x;
        for (int i = 1; i < N; ++i) {
            x = (bb[i] - ss[i - 1] * x) / dd[i];
            o[i] = x;
        }
    } else {
        double x = bb[N - 1] / dd[N - 1];
        o[N - 1] = x;
        for (int i = N - 2; i >= 0; --i) {
            x = (bb[i] - ss[i] * x) / dd[i];
            o[i] = x;
        }
    }
}

// Banded triangular matrices stored by row: lower L[i][i-k] = D[k][i], upper U[i][i+k] =
// D[k][i], k = 0..nd-1, per system D[sys][k][i] (rawkernel.py:34-74 solves, :75-115 products).
__global__ void k_banded_solve(int bsz, int nd, int N, const double* __restrict__ D, const double* __restrict__ b,
                               double* __restrict__ out, int lower) {
    const long long sys = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= bsz) return;
    const double* Dk = D + sys * nd * N;
    const double* bb = b + sys * N;
    double* o = out + sys * N;
    if (lower) {
        for (int i = 0; i < N; ++i) {
            double s = 0.0;
            for (int k = 1; k < nd && k <= i; ++k) s += Dk[(size_t)k * N + i] * o[i - k];
            o[i] = (bb[i] - s) / Dk[i];
        }
    } else {
        for (int i = N - 1; i >= 0; --i) {
            double s = 0.0;
            for (int k = 1; k < nd && i + k < N; ++k) s += Dk[(size_t)k * N + i] * o[i + k];
            o[i] = (bb[i] - s) / Dk[i];
        }
    }
}

__global__ void k_banded_mv(int bsz, int nd, int N, const double* __restrict__ D, const double* __restrict__ b,
                            double* __restrict__ out, int lower) {
    const long long sys = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= bsz) return;
    const double* Dk = D + sys * nd * N;
    const double* bb = b + sys * N;
    double* o = out + sys * N;
    for (int i = 0; i < N; ++i) {
        double s = 0.0;
        if (lower)
            for (int k = 0; k < nd && k <= i; ++k) s += Dk[(size_t)k * N + i] * bb[i - k];
        else
            for (int k = 0; k < nd && i + k < N; ++k) s += Dk[(size_t)k * N + i] * bb[i + k];
        o[i] = s;
    }
}

// One upwind backward-Euler solve (I + a dt D) x = b along a line of N cells. The band
// matrices are stored by column: D_LtoR (lower) has D[i][i-k] = L[k][i-k], D_RtoL (upper)
// D[i][i+k] = R[k][i+k], k = 0..nd-1, shared by all lines. ltr: sweep left to right with
// D_LtoR, else right to left with D_RtoL (rawkernel.py:168-375).
__device__ inline void be_line(const double* __restrict__ L, const double* __restrict__ R, int nd, int N, double a,
                               bool ltr, double dt, const double* __restrict__ b, double* __restrict__ o) {
    const double ad = a * dt;
    if (ltr) {
        for (int i = 0; i < N; ++i) {
            double s = 0.0;
            for (int k = 1; k < nd && k <= i; ++k) s += __ldg(L + (size_t)k * N + (i - k)) * o[i - k];
            o[i] = (b[i] - ad * s) / (1.0 + ad * __ldg(L + i));
        }
    } else {
        for (int i = N - 1; i >= 0; --i) {
            double s = 0.0;
            for (int k = 1; k < nd && i + k < N; ++k) s += __ldg(R + (size_t)k * N + (i + k)) * o[i + k];
            o[i] = (b[i] - ad * s) / (1.0 + ad * __ldg(R + i));
        }
    }
}

// kind 0, v_r lines: b, out (Nx, Nvt, Nr); a = -E[x] cos(theta_j), left to right when a >= 0
//         (rawkernel.py:168-230)
// kind 1, v_theta lines: b, out (Nx, Nr, Nvt); a = E[x] / v_r, left to right when -a >= 0
//         (:232-296)
// kind 2, x lines: b, out (Nr, Nvt, Nx); a = v_r cos(theta_j), left to right when a >= 0
//         (:298-375)
__global__ void k_adv_be(int kind, const double* __restrict__ L, const double* __restrict__ R,
                         const double* __restrict__ c1, const double* __restrict__ c2, double dt,
                         const double* __restrict__ b, double* __restrict__ out, int nd, int Nr, int Nvt, int Nx) {
    const long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int N;
    double a;
    bool ltr;
    if (kind == 0) {
        if (line >= (long long)Nx * Nvt) return;
        N = Nr;
        a = -c1[line / Nvt] * c2[line % Nvt];
        ltr = a >= 0.0;
    } else if (kind == 1) {
        if (line >= (long long)Nx * Nr) return;
        N = Nvt;
        a = c1[line / Nr] / c2[line % Nr];
        ltr = -a >= 0.0;
    } else {
        if (line >= (long long)Nr * Nvt) return;
        N = Nx;
        a = c1[line / Nvt] * c2[line % Nvt];
        ltr = a >= 0.0;
    }
    be_line(L, R, nd, N, a, ltr, dt, b + line * N, out + line * N);
}

// Unit upper block-triangular solve with a BSR matrix (block size bs, nbr block rows, CSR
// structure indptr/indices over blocks, blocks row-major); one CTA per right-hand side
// (rhs-major b, out: nrhs x nbr*bs). Blocks on or below the diagonal are not read: the
// diagonal blocks are taken as identities (BESolver/cuda/spsm_bsr_upper_tri_solve.cu,
// cusparse_spsolve.py with unit_diagonal=True). Block row i: x_i = b_i - sum_{j > i} A_ij x_j,
// the rows of A_ij split over the warps, a row's dot product over the lanes.
__global__ void k_bsr_upper_unit(int nbr, int bs, int nrhs, const double* __restrict__ data,
                                 const int* __restrict__ indptr, const int* __restrict__ indices,
                                 const double* __restrict__ b, double* __restrict__ out) {
    extern __shared__ double xi[];  // bs: the block row being solved
    const int rhs = blockIdx.x;
    if (rhs >= nrhs) return;
    const int n = nbr * bs;
    const double* bb = b + (size_t)rhs * n;
    double* o = out + (size_t)rhs * n;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = nbr - 1; i >= 0; --i) {
        for (int r = threadIdx.x; r < bs; r += blockDim.x) xi[r] = bb[(size_t)i * bs + r];
        __syncthreads();
        for (int e = indptr[i]; e < indptr[i + 1]; ++e) {
            const int j = indices[e];
            if (j <= i) continue;
            const double* A = data + (size_t)e * bs * bs;
            const double* xj = o + (size_t)j * bs;
            for (int r = w; r < bs; r += nw) {
                double s = 0.0;
                for (int c = lane; c < bs; c += 32) s += A[(size_t)r * bs + c] * xj[c];
                for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
                if (lane == 0) xi[r] -= s;
            }
            __syncthreads();
        }
        for (int r = threadIdx.x; r < bs; r += blockDim.x) o[(size_t)i * bs + r] = xi[r];
        __syncthreads();
    }
}

// C = A B (row-major; A M x K, B K x N), FP64, 32 x 32 output tiles through shared memory:
// the op-split step's collision solve PmatC v (bte_1d3v_solver.py:1797).
constexpr int GT = 32;
__global__ void __launch_bounds__(GT * 8)
k_dgemm_nn(int M, int N, int K, const double* __restrict__ A, int lda, const double* __restrict__ B, int ldb,
           double* __restrict__ C, int ldc) {
    __shared__ double As[GT][GT + 1];
    __shared__ double Bs[GT][GT + 1];
    const int tx = threadIdx.x % GT, ty = threadIdx.x / GT;  // 32 x 8 threads, 4 rows each
    const int row0 = blockIdx.y * GT, col = blockIdx.x * GT + tx;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k0 = 0; k0 < K; k0 += GT) {
        for (int r = ty; r < GT; r += 8) {
            const int ar = row0 + r, ak = k0 + tx;
            As[r][tx] = (ar < M && ak < K) ? A[(size_t)ar * lda + ak] : 0.0;
            const int bk = k0 + r;
            Bs[r][tx] = (bk < K && col < N) ? B[(size_t)bk * ldb + col] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < GT; ++kk) {
            const double b = Bs[kk][tx];
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[i] += As[ty + 8 * i][kk] * b;
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = row0 + ty + 8 * i;
        if (r < M && col < N) C[(size_t)r * ldc + col] = acc[i];
    }
}

// out = in with its three axes reordered: in has dims (d0, d1, d2); output axis a is input
// axis perm[a] (the op-split step's layout swaps, bte_1d3v_solver.py:1813,1831,1848).
__global__ void k_permute3(int d0, int d1, int d2, int p0, int p1, int p2, const double* __restrict__ in,
                           double* __restrict__ out) {
    const long long n = (long long)d0 * d1 * d2;
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int dims[3] = {d0, d1, d2};
    const int od1 = dims[p1], od2 = dims[p2];
    const int c = (int)(o % od2), b = (int)((o / od2) % od1), a = (int)(o / ((long long)od1 * od2));
    int idx[3];
    idx[p0] = a;
    idx[p1] = b;
    idx[p2] = c;
    out[o] = in[((long long)idx[0] * d1 + idx[1]) * d2 + idx[2]];
}

// Inflow boundary of the x sweep on v (Nr, Nvt, Nx): zero at the first x point for
// theta_j <= pi/2, at the last for theta_j > pi/2 (bte_1d3v_solver.py:1839-1840).
__global__ void k_fvm_inflow_zero(int Nr, int Nvt, int Nx, const double* __restrict__ vt, double* v) {
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= Nr * Nvt) return;
    const int j = line % Nvt;
    const double half_pi = 0.5 * 3.14159265358979323846;
    v[(size_t)line * Nx + ((vt[j] <= half_pi) ? 0 : Nx - 1)] = 0.0;
}

thread_local std::string g_sw_err;
int sw_fail(const char* msg) {
    g_sw_err = msg;
    return BTE_ERR_ARG;
}
int sw_launched(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return 0;
    g_sw_err = std::string(what) + ": " + cudaGetErrorString(e);
    return BTE_ERR_CUDA;
}

}  // namespace

extern "C" {

const char* bte_sweep_last_error(void) { return g_sw_err.c_str(); }

int bte_bidiag_solve(int bsz, int N, const double* diag, const double* sdiag, const double* b, double* out, int lower,
                     void* stream) {
    if (bsz < 0 || N < 1) return sw_fail("bte_bidiag_solve: bad sizes");
    if (bsz == 0) return 0;
    if (!diag || !b || !out || (N > 1 && !sdiag)) return sw_fail("bte_bidiag_solve: null pointer");
    if (b == out) return sw_fail("bte_bidiag_solve: out must not alias b");
    k_bidiag<<<sw_blocks(bsz), SW_THREADS, 0, (cudaStream_t)stream>>>(bsz, N, diag, sdiag, b, out, lower ? 1 : 0);
    return sw_launched("bte_bidiag_solve");
}

int bte_banded_tri_solve(int bsz, int ndiags, int N, const double* diags, const double* b, double* out, int lower,
                         void* stream) {
    if (bsz < 0 || N < 1 || ndiags < 1) return sw_fail("bte_banded_tri_solve: bad sizes");
    if (bsz == 0) return 0;
    if (!diags || !b || !out) return sw_fail("bte_banded_tri_solve: null pointer");
    if (b == out) return sw_fail("bte_banded_tri_solve: out must not alias b");
    k_banded_solve<<<sw_blocks(bsz), SW_THREADS, 0, (cudaStream_t)stream>>>(bsz, ndiags, N, diags, b, out, lower ? 1 : 0);
    return sw_launched("bte_banded_tri_solve");
}

int bte_banded_tri_mv(int bsz, int ndiags, int N, const double* diags, const double* b, double* out, int lower,
                      void* stream) {
    if (bsz < 0 || N < 1 || ndiags < 1) return sw_fail("bte_banded_tri_mv: bad sizes");
    if (bsz == 0) return 0;
    if (!diags || !b || !out) return sw_fail("bte_banded_tri_mv: null pointer");
    if (b == out) return sw_fail("bte_banded_tri_mv: out must not alias b");
    k_banded_mv<<<sw_blocks(bsz), SW_THREADS, 0, (cudaStream_t)stream>>>(bsz, ndiags, N, diags, b, out, lower ? 1 : 0);
    return sw_launched("bte_banded_tri_mv");
}

int bte_adv_be_sweep(int kind, const double* D_LtoR, const double* D_RtoL, const double* c1, const double* c2,
                     double dt, const double* b, double* out, int ndiags, int Nr, int Nvt, int Nx, void* stream) {
    if (kind < 0 || kind > 2) return sw_fail("bte_adv_be_sweep: kind must be 0 (v_r), 1 (v_theta) or 2 (x)");
    if (Nr < 1 || Nvt < 1 || Nx < 1 || ndiags < 1) return sw_fail("bte_adv_be_sweep: bad sizes");
    if (!D_LtoR || !D_RtoL || !c1 || !c2 || !b || !out) return sw_fail("bte_adv_be_sweep: null pointer");
    if (b == out) return sw_fail("bte_adv_be_sweep: out must not alias b");
    const long long lines = kind == 0 ? (long long)Nx * Nvt : kind == 1 ? (long long)Nx * Nr : (long long)Nr * Nvt;
    k_adv_be<<<sw_blocks(lines), SW_THREADS, 0, (cudaStream_t)stream>>>(kind, D_LtoR, D_RtoL, c1, c2, dt, b, out,
                                                                       ndiags, Nr, Nvt, Nx);
    return sw_launched("bte_adv_be_sweep");
}

int bte_bsr_upper_unit_solve(int nbr, int bs, int nrhs, const double* data, const int* indptr, const int* indices,
                             const double* b, double* out, void* stream) {
    if (nbr < 0 || bs < 1 || nrhs < 0) return sw_fail("bte_bsr_upper_unit_solve: bad sizes");
    if (nbr == 0 || nrhs == 0) return 0;
    if (!data || !indptr || !indices || !b || !out) return sw_fail("bte_bsr_upper_unit_solve: null pointer");
    if (b == out) return sw_fail("bte_bsr_upper_unit_solve: out must not alias b");
    const size_t smem = (size_t)bs * sizeof(double);
    cudaError_t e = bte_raise_smem_limit((const void*)k_bsr_upper_unit, smem);
    if (e != cudaSuccess) return sw_fail("bte_bsr_upper_unit_solve: block too large for shared memory");
    k_bsr_upper_unit<<<nrhs, 256, smem, (cudaStream_t)stream>>>(nbr, bs, nrhs, data, indptr, indices, b, out);
    return sw_launched("bte_bsr_upper_unit_solve");
}

int bte_dgemm_nn(int M, int N, int K, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                 void* stream) {
    if (M < 0 || N < 0 || K < 0 || lda < K || ldb < N || ldc < N) return sw_fail("bte_dgemm_nn: bad sizes");
    if (M == 0 || N == 0) return 0;
    if (!A || !B || !C) return sw_fail("bte_dgemm_nn: null pointer");
    if (C == A || C == B) return sw_fail("bte_dgemm_nn: C must not alias A or B");
    dim3 grid((unsigned)((N + GT - 1) / GT), (unsigned)((M + GT - 1) / GT));
    k_dgemm_nn<<<grid, GT * 8, 0, (cudaStream_t)stream>>>(M, N, K, A, lda, B, ldb, C, ldc);
    return sw_launched("bte_dgemm_nn");
}

int bte_permute3(int d0, int d1, int d2, int p0, int p1, int p2, const double* in, double* out, void* stream) {
    if (d0 < 0 || d1 < 0 || d2 < 0) return sw_fail("bte_permute3: bad sizes");
    const int s = (1 << p0) | (1 << p1) | (1 << p2);
    if (p0 < 0 || p1 < 0 || p2 < 0 || p0 > 2 || p1 > 2 || p2 > 2 || s != 7) return sw_fail("bte_permute3: perm must reorder 0, 1, 2");
    const long long n = (long long)d0 * d1 * d2;
    if (n == 0) return 0;
    if (!in || !out || in == out) return sw_fail("bte_permute3: null or aliased buffers");
    k_permute3<<<sw_blocks(n), SW_THREADS, 0, (cudaStream_t)stream>>>(d0, d1, d2, p0, p1, p2, in, out);
    return sw_launched("bte_permute3");
}

int bte_fvm_inflow_zero(int Nr, int Nvt, int Nx, const double* vt, double* v, void* stream) {
    if (Nr < 1 || Nvt < 1 || Nx < 1) return sw_fail("bte_fvm_inflow_zero: bad sizes");
    if (!vt || !v) return sw_fail("bte_fvm_inflow_zero: null pointer");
    k_fvm_inflow_zero<<<sw_blocks((long long)Nr * Nvt), SW_THREADS, 0, (cudaStream_t)stream>>>(Nr, Nvt, Nx, vt, v);
    return sw_launched("bte_fvm_inflow_zero");
}

}  // extern "C"
