/* C ABI of the 1D3V step (spectral v-space x discrete ordinates x Chebyshev collocation in x)
 * of the GB300 velocity-space library. Counterpart of the spectral path of the reference's
 * bte_1d3v (BESolver/python/bte_1d3v_solver.py:218-2244); the Python class
 * boltzmann_gb300.bte_1d3v builds the setup operators and calls these entry points.
 *
 * Layouts (device, double): ordinates V[(r * Nvt + j) * Nx + x] (the reference's (Nr * Nvt, Nx)
 * array); v-space U[x * n + r * nsh + l], n = Nr * nsh (x-major: one point's coefficients
 * contiguous). Every entry point returns 0 or a negative BTE_ERR_* code; bte1d_last_error()
 * gives the message. One handle is used by one stream at a time. */
#ifndef BTE1D_GB300_H
#define BTE1D_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct Bte1d bte1d;

/* Create a 1D3V handle on `device` from host setup operators:
 *   Q, Qinv [Nr x Nr], d [Nr]   eigendecomposition of the radial x-advection operator
 *                                adv_x = M_r^-1 vth (tau / L) int v^3 phi_p phi_k
 *                                (bte_1d3v_solver.py:621-625, op_adv_x_q / _qinv / _d)
 *   cos_theta [Nvt]             ordinate directions (spec_spherical.py:1020-1064, gl_vt)
 *   D [Nx x Nx]                 Chebyshev collocation derivative (collocation_op.py:8-33)
 *   po2sh [nsh x Nvt], psh2o [Nvt x nsh]  ordinate <-> harmonic projections
 *                                (spec_spherical.py:997-1008, op_po2sh / op_psh2o)
 *   Cv, Av [n x n]              tau n0 np0 (C_en + Tg C_gT) and tau A_v, M^-1-scaled
 *                                (bte_1d3v_solver.py:1051-1055, Lmat_mvec)
 *   restart                     GMRES restart length (params gmres_rsrt). */
int bte1d_create(int device, int Nr, int nsh, int Nvt, int Nx, const double* Q, const double* Qinv, const double* d,
                 const double* cos_theta, const double* D, const double* po2sh, const double* psh2o,
                 const double* Cv, const double* Av, int restart, bte1d** out);
int bte1d_destroy(bte1d* h);

/* x-advection over a backward-Euler step of size h, V in place (ordinates layout).
 * Replaces bte_1d3v.step_bte_x (bte_1d3v_solver.py:912-982) with the BE Chebyshev operators
 * of __initialize_bte_adv_x__ (:780-887); the Nr * Nvt systems are factored once per h. */
int bte1d_step_x(bte1d* h, double hstep, double* V, void* stream);

/* v-space step of size dt at field E [Nx], V in place (ordinates layout): GMRES on
 * Lmat_mvec with a per-point block preconditioner. info4 (host) = {iterations, ||r||,
 * ||r|| / ||b||, 0 converged / 1 not}.
 * Replaces bte_1d3v.step_bte_v (bte_1d3v_solver.py:984-1137). */
int bte1d_step_v(bte1d* h, double dt, const double* E, double* V, double rtol, double atol, int max_iter,
                 double* info4, void* stream);

/* Y = X - dt (Cv X + E (Av X)) per point, x-major v-space layout (Lmat_mvec,
 * bte_1d3v_solver.py:1051-1055). */
int bte1d_lmat(bte1d* h, double dt, const double* E, const double* X, double* Y, void* stream);

/* Block preconditioner of the v-step: Y = B_x^-1 X per point, B_x = I - dt (Cv + E_x Av)
 * factored in FP32 (x-major v-space layout). The reference's Mmat_mvec applies the inverse of
 * the nearest of num_pc_ops E values instead (bte_1d3v_solver.py:889-910,1057-1064). */
int bte1d_block_solve(bte1d* h, double dt, const double* E, const double* X, double* Y, void* stream);

/* ordinates <-> spherical harmonics (ords_to_sph / sph_to_ords, bte_1d3v_solver.py:678-694);
 * U in the x-major v-space layout. */
int bte1d_ords_to_lm(bte1d* h, const double* V, double* U, void* stream);
int bte1d_lm_to_ords(bte1d* h, const double* U, double* V, void* stream);

/* The backward-Euler operator of the fully implicit spectral step on ordinates (layout above):
 *   Y = V - dt (P_sh2o (Cv + E_x Av) P_o2sh V - (adv_x (x) diag(cos theta_j)) V D_X^T)
 * with D_X the upwinded Chebyshev derivative (D_L for cos(theta_j) >= 0, D_R otherwise) and
 * identity rows on the inflow boundary. The reference has no fully implicit solver for the
 * spectral v-space (bte_1d3v_solver.py:1891 asserts the finite-volume one); this operator is
 * composed from its operators as its matvec test composes them (test_bte_1d_matvec.py:19-83):
 * Lmat_mvec (bte_1d3v_solver.py:1051-1055) plus step_bte_x's BE Chebyshev advection (:912-982). */
int bte1d_fim_matvec(bte1d* h, double dt, const double* E, const double* V, double* Y, void* stream);

/* One fully implicit step of size dt at field E [Nx]: V <- the solution of
 * bte1d_fim_matvec(V_new) = V with the inflow values of the right-hand side set to 0, by
 * right-preconditioned restarted GMRES (restart = the handle's, utils.py:1172-1262) to
 * ||r|| <= max(atol, rtol ||b||). pc 0: the preconditioner is a Lie split, the exact per-point
 * v-space inverse (FP32 block factors) followed by the backward-Euler x-advection over dt;
 * pc 1: the v-space blocks alone. info4 (host) = {iterations, ||r||, ||r|| / ||b||,
 * 0 converged / 1 not}. */
int bte1d_step_fim(bte1d* h, double dt, const double* E, double* V, double rtol, double atol, int max_iter, int pc,
                   double* info4, void* stream);

/* Kernel launches made through this handle since it was created. */
long long bte1d_launches(const bte1d* h);

/* Last error message of the 1D3V entry points (never NULL). */
const char* bte1d_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
