// Batched FP32 LU with partial pivoting whose trailing updates run on the tcgen05 tensor
// cores (kind::tf32, accumulators in tensor memory), with split-TF32 operands so that the
// factors keep FP32 accuracy.
//
// Replaces, like lu.cu, the explicit batched inverse of the Newton Jacobian
// (xp.linalg.inv in bte_0d3v_batched.py:856-880, applied at :933-934). Same storage
// convention as lu.cu: row-major A[r * ld + c] with NC = N or N + 1 columns (the right-hand
// side appended as column N is eliminated with the matrix), rows never exchanged in
// memory, perm[position] = stored row, info = first zero pivot (1-based), 0 if none.
//
// One CTA per matrix, right-looking by 32-column panels:
//   1. panel: the 32 columns of positions k0..N-1 are held in registers (thread t owns
//      positions k0 + t + i * 256); each column costs one barrier: every warp publishes its
//      best candidate row in shared memory, all threads pick the same winner (largest |a|,
//      lowest position on ties, as LAPACK's i?amax), swap it with position j by registers
//      and apply the rank-one update;
//   2. U12 = L11^-1 A12 for the 32 pivot rows, one thread per column;
//   3. A22 -= L21 U12 in tiles of 128 columns x 128 rows: U12^T (M = 128 columns) and L21
//      (N = 128 rows) are staged in shared memory in the canonical K-major layout (8 x 16 B
//      core matrices, no swizzle), split into a TF32 high part and an FP32 remainder, and
//      one thread issues 4 k-steps x 3 products (hi*hi + hi*lo + lo*hi) of
//      tcgen05.mma.cta_group::1.kind::tf32 into a 128-lane x 128-column TMEM accumulator.
//      The epilogue reads it back with tcgen05.ld (lane = column, so a warp's 32 lanes are
//      32 consecutive columns of one row: coalesced) and updates A22 in global memory,
//      which stays L2-resident while the CTA works on it.
// The split: hi = tf32(x) (round to nearest), lo = x - hi (exact in FP32); hi*hi is exact
// in the FP32 accumulator, the dropped lo*lo term is below 2^-22 |x y|.
#include <cstdint>
#include <climits>
#include "bte_common.cuh"

namespace {

constexpr int TC_NT = 256;         // threads per CTA of the widest variant (8 warps; also 128)
constexpr int TC_NW = TC_NT / 32;  // shared-memory slots for the warps' pivot candidates
constexpr int TC_NB = 32;          // panel width = K of one block step
constexpr int TC_TM = 128;         // trailing columns per tile: MMA M, TMEM lanes
constexpr int TC_TR = 128;         // trailing rows per tile: MMA N, TMEM columns
constexpr uint32_t TC_TMEM_COLS = 128;
constexpr int TC_TILE_BYTES = TC_TM * TC_NB * 4;   // one operand part: 16 KB (TM == TR)
constexpr int TC_L11_LD = TC_NB + 4;        // L11 stored transposed, 16-byte rows
constexpr int TC_CAND_LD = TC_NB + 4;              // a candidate row + key + slot, 16-byte rows
constexpr uint32_t TC_WAIT_LIMIT = 1u << 22;       // bounded wait for an MMA commit

// shared memory map (bytes from the 1024-aligned dynamic base)
constexpr int SM_A_HI = 0;
constexpr int SM_A_LO = SM_A_HI + TC_TILE_BYTES;
constexpr int SM_B_HI = SM_A_LO + TC_TILE_BYTES;
constexpr int SM_B_LO = SM_B_HI + TC_TILE_BYTES;
constexpr int SM_L11 = SM_B_LO + TC_TILE_BYTES;
constexpr int SM_CAND = SM_L11 + ((TC_NB * TC_L11_LD * 4 + 15) & ~15);
constexpr int SM_JBUF = SM_CAND + 2 * TC_NW * TC_CAND_LD * 4;
constexpr int SM_PERM = SM_JBUF + 2 * TC_NB * 4;
__host__ __device__ inline size_t tc_smem_bytes(int N) { return (size_t)SM_PERM + (size_t)N * 4 + 1024; }

// byte offset of element (row m, k) in a [rows x 32] TF32 tile, K-major, no swizzle:
// core matrix (m / 8, k / 4) at (m / 8) * 1024 + (k / 4) * 128, rows of a core matrix 16 B apart
__device__ inline int op_off(int m, int k) { return (m >> 3) * 1024 + (k >> 2) * 128 + (m & 7) * 16 + (k & 3) * 4; }

__device__ inline uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (tcgen05): start address >> 4 (bits 0-13), leading byte
// offset >> 4 (bits 16-29: next core matrix along K), stride byte offset >> 4 (bits 32-45:
// next 8-row group), descriptor version 1 (bits 46-47), base offset 0, no swizzle (61-63)
__device__ inline uint64_t op_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// instruction descriptor of kind::tf32: D F32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12
// = 2), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ inline void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ inline void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}
__device__ inline void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ inline void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ inline void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ inline void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ inline bool mbar_try_wait(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}

// tensor-memory allocation, one full warp
__device__ inline void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ inline void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive TMEM columns of the warp's 32 lanes (lane i of the warp reads TMEM lane
// base + i): v[c] = D[lane][col + c]
__device__ inline void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ inline float tf32_rn(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// four values of one operand row (m, k..k+3) as high and low parts
__device__ inline void put_split4(unsigned char* sm, int m, int k, float a, float b, float c, float d) {
    float4 hi = make_float4(tf32_rn(a), tf32_rn(b), tf32_rn(c), tf32_rn(d));
    float4 lo = make_float4(a - hi.x, b - hi.y, c - hi.z, d - hi.w);
    const int o = op_off(m, k);
    *reinterpret_cast<float4*>(sm + o) = hi;
    *reinterpret_cast<float4*>(sm + TC_TILE_BYTES + o) = lo;
}

template <int ROWS, int OCC, int NT>
__global__ void __launch_bounds__(NT, OCC)
k_lu_tc(int N, int NC, float* __restrict__ A, int ld, long long stride, int32_t* __restrict__ perm_out,
        int32_t* __restrict__ info, int vec4) {
    extern __shared__ unsigned char smraw[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fault;
    // 1024-aligned base for the operand tiles
    unsigned char* sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    float* L11 = reinterpret_cast<float*>(sm + SM_L11);
    float* cand = reinterpret_cast<float*>(sm + SM_CAND);
    float* jbuf = reinterpret_cast<float*>(sm + SM_JBUF);
    int* perm = reinterpret_cast<int*>(sm + SM_PERM);

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    float* a = A + (size_t)blockIdx.x * stride;
    for (int r = tid; r < N; r += NT) perm[r] = r;
    const uint32_t mb = smem_u32(&mbar);
    if (tid == 0) {
        mbar_init(mb, 1);
        s_fault = 0;
    }
    if (wid == 0) tmem_alloc(smem_u32(&tmem_slot), TC_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_slot;
    uint32_t phase = 0;
    int inf = 0;

    for (int k0 = 0; k0 < N; k0 += TC_NB) {
        const int mrows = N - k0;
        const int kb = min(TC_NB, mrows);
        const int ncol = min(TC_NB, NC - k0);
        // ---- 1. panel: positions k0.., columns k0..k0+31 in registers
        float pr[ROWS][TC_NB];
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            const int s = tid + i * NT;
            const float* row = a + (size_t)perm[k0 + min(s, mrows - 1)] * ld + k0;
            if (vec4 && ncol == TC_NB) {
#pragma unroll
                for (int c = 0; c < TC_NB; c += 4) {
                    float4 v = (s < mrows) ? *reinterpret_cast<const float4*>(row + c) : make_float4(0.f, 0.f, 0.f, 0.f);
                    pr[i][c] = v.x; pr[i][c + 1] = v.y; pr[i][c + 2] = v.z; pr[i][c + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int c = 0; c < TC_NB; ++c) pr[i][c] = (s < mrows && c < ncol) ? row[c] : 0.f;
            }
        }
#pragma unroll
        for (int j = 0; j < TC_NB; ++j) {
            if (j >= kb) break;
            const int par = j & 1;
            float* cb = cand + par * TC_NW * TC_CAND_LD;
            float* jb = jbuf + par * TC_NB;
            if (tid == j) {
#pragma unroll
                for (int c = 0; c < TC_NB; c += 4)
                    *reinterpret_cast<float4*>(jb + c) = make_float4(pr[0][c], pr[0][c + 1], pr[0][c + 2], pr[0][c + 3]);
            }
            // the thread's best candidate among positions >= j: largest |a| (NaN counts as 0)
            uint32_t bkey = 0;
            int bs = INT_MAX;
#pragma unroll
            for (int i = 0; i < ROWS; ++i) {
                const int s = tid + i * NT;
                if (s >= j && s < mrows) {
                    const float v = fabsf(pr[i][j]);
                    const uint32_t key = (v == v) ? __float_as_uint(v) : 0u;
                    if (bs == INT_MAX || key > bkey) { bkey = key; bs = s; }
                }
            }
            const uint32_t kmax = __reduce_max_sync(0xffffffffu, bkey);
            const uint32_t smin =
                __reduce_min_sync(0xffffffffu, (bs != INT_MAX && bkey == kmax) ? (uint32_t)bs : 0xffffffffu);
            float* myc = cb + wid * TC_CAND_LD;
            if (smin != 0xffffffffu && (uint32_t)bs == smin) {
#pragma unroll
                for (int i = 0; i < ROWS; ++i)
                    if (tid + i * NT == bs) {
#pragma unroll
                        for (int c = 0; c < TC_NB; c += 4)
                            *reinterpret_cast<float4*>(myc + c) =
                                make_float4(pr[i][c], pr[i][c + 1], pr[i][c + 2], pr[i][c + 3]);
                    }
                reinterpret_cast<uint32_t*>(myc)[TC_NB] = kmax;
                reinterpret_cast<int*>(myc)[TC_NB + 1] = bs;
            } else if (smin == 0xffffffffu && lane == 0) {
                reinterpret_cast<int*>(myc)[TC_NB + 1] = INT_MAX;
            }
            __syncthreads();
            // the same winner in every thread: (key, slot) pairs read 8 bytes at a time
            uint32_t K = 0;
            int S = INT_MAX, W = 0;
#pragma unroll
            for (int w2 = 0; w2 < NT / 32; ++w2) {
                const uint2 ks = *reinterpret_cast<const uint2*>(cb + w2 * TC_CAND_LD + TC_NB);
                const int s2 = (int)ks.y;
                if (s2 != INT_MAX && (S == INT_MAX || ks.x > K || (ks.x == K && s2 < S))) { K = ks.x; S = s2; W = w2; }
            }
            const float* prow = cb + W * TC_CAND_LD;
            // the pivot row's columns j.. in registers (16-byte loads from the 4-aligned start)
            float pv[TC_NB];
#pragma unroll
            for (int c = (j & ~3); c < TC_NB; c += 4) {
                const float4 v = *reinterpret_cast<const float4*>(prow + c);
                pv[c] = v.x; pv[c + 1] = v.y; pv[c + 2] = v.z; pv[c + 3] = v.w;
            }
            if (S != j && S != INT_MAX) {
                if (tid == j) {
#pragma unroll
                    for (int c = 0; c < TC_NB; c += 4) {
                        const float4 v = *reinterpret_cast<const float4*>(prow + c);
                        pr[0][c] = v.x; pr[0][c + 1] = v.y; pr[0][c + 2] = v.z; pr[0][c + 3] = v.w;
                    }
                }
#pragma unroll
                for (int i = 0; i < ROWS; ++i)
                    if (tid + i * NT == S) {
#pragma unroll
                        for (int c = 0; c < TC_NB; c += 4) {
                            const float4 v = *reinterpret_cast<const float4*>(jb + c);
                            pr[i][c] = v.x; pr[i][c + 1] = v.y; pr[i][c + 2] = v.z; pr[i][c + 3] = v.w;
                        }
                    }
                if (tid == 0) {
                    const int t = perm[k0 + j];
                    perm[k0 + j] = perm[k0 + S];
                    perm[k0 + S] = t;
                }
            }
            const float d = pv[j];
            if (tid == 0 && !(d != 0.f) && inf == 0) inf = k0 + j + 1;
            const float inv = (d != 0.f) ? __frcp_rn(d) : 0.f;
#pragma unroll
            for (int i = 0; i < ROWS; ++i) {
                const int s = tid + i * NT;
                if (s > j && s < mrows) {
                    const float l = pr[i][j] * inv;
                    pr[i][j] = l;
#pragma unroll
                    for (int c = j + 1; c < TC_NB; ++c) pr[i][c] -= l * pv[c];
                }
            }
        }
        __syncthreads();  // perm of this panel final
        // write the panel back (each position's data returns to its own stored row) and L11
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            const int s = tid + i * NT;
            if (s < mrows) {
                float* row = a + (size_t)perm[k0 + s] * ld + k0;
                if (vec4 && ncol == TC_NB) {
#pragma unroll
                    for (int c = 0; c < TC_NB; c += 4)
                        *reinterpret_cast<float4*>(row + c) = make_float4(pr[i][c], pr[i][c + 1], pr[i][c + 2], pr[i][c + 3]);
                } else {
#pragma unroll
                    for (int c = 0; c < TC_NB; ++c)
                        if (c < ncol) row[c] = pr[i][c];
                }
                if (i == 0 && s < TC_NB) {
#pragma unroll
                    for (int c = 0; c < TC_NB; ++c) L11[c * TC_L11_LD + s] = pr[0][c];
                }
            }
        }
        const int ncols = NC - k0 - TC_NB;   // columns right of the panel (> 0 implies kb == 32)
        const int nrows = N - k0 - TC_NB;    // trailing rows
        if (ncols <= 0) break;
        __syncthreads();
        // ---- 2. U12 = L11^-1 A12, one thread per column
        for (int c = tid; c < ncols; c += NT) {
            float x[TC_NB];
#pragma unroll
            for (int j = 0; j < TC_NB; ++j) x[j] = a[(size_t)perm[k0 + j] * ld + k0 + TC_NB + c];
#pragma unroll
            for (int i = 0; i < TC_NB; ++i) {
                // keeps the compiler from hoisting all 496 multipliers into registers
                asm volatile("" ::: "memory");
                float lc[TC_NB];
#pragma unroll
                for (int j = ((i + 1) & ~3); j < TC_NB; j += 4) {
                    const float4 v = *reinterpret_cast<const float4*>(L11 + i * TC_L11_LD + j);
                    lc[j] = v.x; lc[j + 1] = v.y; lc[j + 2] = v.z; lc[j + 3] = v.w;
                }
#pragma unroll
                for (int j = i + 1; j < TC_NB; ++j) x[j] -= lc[j] * x[i];
            }
#pragma unroll
            for (int j = 0; j < TC_NB; ++j) a[(size_t)perm[k0 + j] * ld + k0 + TC_NB + c] = x[j];
        }
        if (nrows <= 0) break;  // last panel
        __syncthreads();
        // ---- 3. A22 -= L21 U12 on the tensor cores
        for (int g0 = 0; g0 < nrows; g0 += TC_TR) {
            // B operand: L21 rows g0.., K = the panel's 32 columns
            for (int e = tid; e < TC_TR * (TC_NB / 4); e += NT) {
                const int r = e >> 3, k = (e & 7) * 4;
                float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
                if (g0 + r < nrows) {
                    const float* row = a + (size_t)perm[k0 + TC_NB + g0 + r] * ld + k0 + k;
                    if (vec4) {
                        float4 v = *reinterpret_cast<const float4*>(row);
                        v0 = v.x; v1 = v.y; v2 = v.z; v3 = v.w;
                    } else {
                        v0 = row[0]; v1 = row[1]; v2 = row[2]; v3 = row[3];
                    }
                }
                put_split4(sm + SM_B_HI, r, k, v0, v1, v2, v3);
            }
            for (int c0 = 0; c0 < ncols; c0 += TC_TM) {
                // A operand: U12^T, row m = column c0 + m of U12, k = pivot row
                for (int e = tid; e < TC_TM * (TC_NB / 4); e += NT) {
                    const int m = e & (TC_TM - 1), k = (e >> 7) * 4;
                    float v[4] = {0.f, 0.f, 0.f, 0.f};
                    if (c0 + m < ncols) {
#pragma unroll
                        for (int q = 0; q < 4; ++q) v[q] = a[(size_t)perm[k0 + k + q] * ld + k0 + TC_NB + c0 + m];
                    }
                    put_split4(sm + SM_A_HI, m, k, v[0], v[1], v[2], v[3]);
                }
                fence_async_smem();
                tc_fence_before();
                __syncthreads();
                if (tid == 0) {
                    tc_fence_after();
                    const uint32_t ahi = smem_u32(sm + SM_A_HI), alo = smem_u32(sm + SM_A_LO);
                    const uint32_t bhi = smem_u32(sm + SM_B_HI), blo = smem_u32(sm + SM_B_LO);
                    constexpr uint32_t idesc = idesc_tf32(TC_TM, TC_TR);
#pragma unroll
                    for (int ks = 0; ks < TC_NB / 8; ++ks) {
                        const uint32_t o = ks * 256;
                        mma_tf32(tbase, op_desc(alo + o), op_desc(bhi + o), idesc, ks > 0 ? 1u : 0u);
                        mma_tf32(tbase, op_desc(ahi + o), op_desc(blo + o), idesc, 1u);
                        mma_tf32(tbase, op_desc(ahi + o), op_desc(bhi + o), idesc, 1u);
                    }
                    mma_commit(mb);
                    uint32_t it = 0;
                    while (!mbar_try_wait(mb, phase))
                        if (++it > TC_WAIT_LIMIT) { s_fault = 1; break; }
                }
                phase ^= 1u;
                __syncthreads();
                tc_fence_after();
                if (s_fault) break;
                // epilogue: warp w reads TMEM lanes 32 (w % 4).. (columns) and its share of
                // the TMEM columns (rows): all 128 with 4 warps, 64 (w / 4).. with 8
                {
                    constexpr int RH = TC_TR / (NT / 128);
                    const int q = wid & 3, h = wid >> 2;
                    const int m = 32 * q + lane;
                    const bool colok = (c0 + m) < ncols;
                    float* colp = a + k0 + TC_NB + c0 + m;
#pragma unroll 1
                    for (int r0 = RH * h; r0 < RH * h + RH; r0 += 16) {
                        if (g0 + r0 >= nrows) break;  // warp-uniform
                        float dv[16];
                        tmem_ld16(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)r0, dv);
                        float old[16];
                        int rowoff[16];
#pragma unroll
                        for (int t = 0; t < 16; ++t) {
                            const int r = g0 + r0 + t;
                            rowoff[t] = (r < nrows) ? perm[k0 + TC_NB + r] * ld : -1;
                        }
#pragma unroll
                        for (int t = 0; t < 16; ++t) old[t] = (colok && rowoff[t] >= 0) ? colp[rowoff[t]] : 0.f;
#pragma unroll
                        for (int t = 0; t < 16; ++t)
                            if (colok && rowoff[t] >= 0) colp[rowoff[t]] = old[t] - dv[t];
                    }
                }
                tc_fence_before();
                __syncthreads();  // TMEM and the operand tiles are free again
            }
            if (s_fault) break;
        }
        if (s_fault) break;
        __syncthreads();
    }
    if (s_fault) {
        // an MMA commit never arrived: wait once more (bounded) before giving TMEM back
        if (tid == 0) {
            uint32_t it = 0;
            while (!mbar_try_wait(mb, phase) && ++it < TC_WAIT_LIMIT) {}
        }
        __syncthreads();
    }
    for (int r = tid; r < N; r += NT) perm_out[(size_t)blockIdx.x * N + r] = perm[r];
    if (tid == 0) info[blockIdx.x] = s_fault ? -1 : inf;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (wid == 0) tmem_dealloc(tbase, TC_TMEM_COLS);
}

template <int ROWS, int OCC, int NT>
cudaError_t launch_tc(int P, int N, int NC, float* A, int ld, long long stride, int32_t* piv, int32_t* info,
                      cudaStream_t s) {
    const size_t sm = tc_smem_bytes(N);
    cudaError_t e = bte_raise_smem_limit((const void*)k_lu_tc<ROWS, OCC, NT>, sm);
    if (e != cudaSuccess) return e;
    const int vec4 = (ld % 4 == 0 && stride % 4 == 0 && ((uintptr_t)A & 15) == 0) ? 1 : 0;
    k_lu_tc<ROWS, OCC, NT><<<P, NT, sm, s>>>(N, NC, A, ld, stride, piv, info, vec4);
    return cudaGetLastError();
}

}  // namespace

// largest N the tensor-core kernel takes (its panel is two 32-column rows per thread)
int bte_lu_tc_max_n() { return 2 * TC_NT; }

// variant 0: 256 threads, two CTAs per SM (the registers of two, 2 x 128 tensor-memory
// columns); 1: 256 threads, one CTA per SM (half the matrices in flight, so that their
// trailing updates stay in L2); 2: 128 threads (4 warps: half the per-column pivot-search work
// per matrix, up to four panel rows per thread), two CTAs per SM
cudaError_t bte_lu_factor_tc(int P, int N, int NC, float* A, int ld, long long stride, int32_t* piv, int32_t* info,
                             cudaStream_t s, int variant) {
    if (P <= 0) return cudaSuccess;
    if (N < 1 || N > 2 * TC_NT || NC < N || NC > N + 1 || ld < NC) return cudaErrorInvalidValue;
    if ((long long)N * ld >= (1ll << 31)) return cudaErrorInvalidValue;  // row offsets are 32-bit
    if (variant == 2) {
        if (N <= 128) return launch_tc<1, 2, 128>(P, N, NC, A, ld, stride, piv, info, s);
        if (N <= 256) return launch_tc<2, 2, 128>(P, N, NC, A, ld, stride, piv, info, s);
        if (N <= 384) return launch_tc<3, 2, 128>(P, N, NC, A, ld, stride, piv, info, s);
        return launch_tc<4, 2, 128>(P, N, NC, A, ld, stride, piv, info, s);
    }
    if (variant == 1) {
        if (N <= TC_NT) return launch_tc<1, 1, 256>(P, N, NC, A, ld, stride, piv, info, s);
        return launch_tc<2, 1, 256>(P, N, NC, A, ld, stride, piv, info, s);
    }
    if (N <= TC_NT) return launch_tc<1, 2, 256>(P, N, NC, A, ld, stride, piv, info, s);
    return launch_tc<2, 2, 256>(P, N, NC, A, ld, stride, piv, info, s);
}
