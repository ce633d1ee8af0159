/* C ABI of the batched banded kernels of the 1D3V finite-volume path (double precision,
 * device pointers, caller-owned buffers). Counterparts of the reference's CuPy raw kernels
 * (BESolver/python/rawkernel.py) and BSR triangular solve (BESolver/cuda/
 * spsm_bsr_upper_tri_solve.cu, BESolver/python/cusparse_spsolve.py), with the same array
 * layouts. Every entry point returns 0 or a negative BTE_ERR_* code (bte_gb300.h);
 * bte_sweep_last_error() gives the message. `out` never aliases `b`. */
#ifndef BTE_SWEEPS_GB300_H
#define BTE_SWEEPS_GB300_H
#ifdef __cplusplus
extern "C" {
#endif

/* bsz bidiagonal systems of size N: diag [bsz x N], sdiag [bsz x (N-1)] (the sub-diagonal
 * when lower, the super-diagonal otherwise), b, out [bsz x N].
 * Replaces rawkernel.bidiagonal_solve_batched (rawkernel.py:5-33,389-413). */
int bte_bidiag_solve(int bsz, int N, const double* diag, const double* sdiag, const double* b, double* out, int lower,
                     void* stream);

/* bsz banded triangular systems stored by row: diags [bsz x ndiags x N], lower
 * L[i][i-k] = diags[k][i], upper U[i][i+k] = diags[k][i]; solve L x = b (or U x = b).
 * Replaces rawkernel.banded_tri_solve_batched (rawkernel.py:34-74,415-439). */
int bte_banded_tri_solve(int bsz, int ndiags, int N, const double* diags, const double* b, double* out, int lower,
                         void* stream);

/* out = L b (or U b) with the banded triangular matrices of bte_banded_tri_solve.
 * Replaces rawkernel.banded_tri_mv_batched (rawkernel.py:75-115,441-466). */
int bte_banded_tri_mv(int bsz, int ndiags, int N, const double* diags, const double* b, double* out, int lower,
                      void* stream);

/* Upwind backward-Euler advection solves (I + a dt D) x = b along lines, the band matrices
 * stored by column and shared by all lines: D_LtoR [ndiags x N] with D[i][i-k] =
 * D_LtoR[k][i-k], D_RtoL [ndiags x N] with D[i][i+k] = D_RtoL[k][i+k].
 *   kind 0 (v_r):     b, out (Nx, Nvt, Nr), N = Nr,  a = -c1[x] c2[j] (c1 = E, c2 = cos theta),
 *                     left to right when a >= 0        replaces rawkernel.adv_vr_BE (:168-230,468-479)
 *   kind 1 (v_theta): b, out (Nx, Nr, Nvt), N = Nvt, a = c1[x] / c2[r] (c1 = E, c2 = v_r),
 *                     left to right when -a >= 0       replaces rawkernel.adv_vt_BE (:232-296,481-492)
 *   kind 2 (x):       b, out (Nr, Nvt, Nx), N = Nx,  a = c1[r] c2[j] (c1 = v_r, c2 = cos theta),
 *                     left to right when a >= 0        replaces rawkernel.adv_x_BE (:298-375,494-505) */
int bte_adv_be_sweep(int kind, const double* D_LtoR, const double* D_RtoL, const double* c1, const double* c2,
                     double dt, const double* b, double* out, int ndiags, int Nr, int Nvt, int Nx, void* stream);

/* Unit upper block-triangular solve with a BSR matrix: nbr block rows of bs x bs blocks,
 * row-major blocks data [nnzb x bs x bs], CSR structure over blocks indptr [nbr + 1],
 * indices [nnzb] (int32); blocks on or below the diagonal are ignored (unit diagonal).
 * b, out [nrhs x nbr*bs], one right-hand side per row.
 * Replaces the reference's spsm_bsr_upper_tri_solve kernel and cusparse_spsolve.SpSMSolver
 * with lower=False, unit_diagonal=True (spsm_bsr_upper_tri_solve.cu:1-61). */
int bte_bsr_upper_unit_solve(int nbr, int bs, int nrhs, const double* data, const int* indptr, const int* indices,
                             const double* b, double* out, void* stream);

/* C = A B, row-major FP64 (A M x K with row stride lda, B K x N, C M x N); C aliases neither.
 * The op-split step's dense collision solve PmatC v (bte_1d3v_solver.py:1797). */
int bte_dgemm_nn(int M, int N, int K, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                 void* stream);

/* out = in with its axes reordered: in (d0, d1, d2) contiguous; output axis a is input axis
 * p_a (a permutation of 0, 1, 2). The op-split step's xp.swapaxes layout changes
 * (bte_1d3v_solver.py:1813,1831,1848). */
int bte_permute3(int d0, int d1, int d2, int p0, int p1, int p2, const double* in, double* out, void* stream);

/* Inflow boundary of the x sweep on v (Nr, Nvt, Nx): v[r][j][0] = 0 where vt[j] <= pi/2 and
 * v[r][j][Nx-1] = 0 where vt[j] > pi/2 (bte_1d3v_solver.py:1839-1840). */
int bte_fvm_inflow_zero(int Nr, int Nvt, int Nx, const double* vt, double* v, void* stream);

const char* bte_sweep_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
