/* C ABI of the finite-volume 1D3V fully implicit step (double precision). Set-up arrays are
 * host pointers, copied at the call; E, X, Y and V are device pointers. Every entry point
 * returns 0 or a negative BTE_ERR_* code (bte_gb300.h); bte_fvm_last_error() gives the message.
 *
 * Layout: v[(r * Nvt + j) * Nx + x], r the radial cell, j the ordinate, x the spatial point
 * (the reference's (Nr * Nvt, Nx) array). Band arrays are the op-split sweeps' column-stored
 * bands (nd, N): lower D[i][i-k] = B[k][i-k], upper D[i][i+k] = B[k][i+k]; the v_theta bands
 * carry the sin(theta) factor.
 *
 * Replaces, in BESolver/python/bte_1d3v_solver.py: the fully implicit branch of step()
 * (:1890-2009) with rhs_mvec (:1915-1955) and its op-split preconditioner
 * (step_op_split, :1745-1870); the dense collision inverse PmatC of init() (:1346-1375) is
 * passed in factored form; the semi-Lagrangian step (:2024-2027, step_adv_vx_sl :2244-2314). */
#ifndef BTE_FVM_GB300_H
#define BTE_FVM_GB300_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct bte_fvm bte_fvm;

/* dt: the step; dtx: the step size the x-shift operator is set up with (init(dt),
 * bte_1d3v_solver.py:1401); tau = 1 / frequency; kappa = n0 np0; cA = qe / (me vth);
 * ax = vth tau / L. */
typedef struct bte_fvm_coef {
    double dt, dtx, tau, kappa, cA, ax;
} bte_fvm_coef;

/* Grids vr [Nr] (cell centres, units of vth, > 0), vt [Nvt] (ordinates, Nvt even),
 * w [Nvt] (2 pi times the ordinate weights); the collision operator
 * C = gain (x) (1 w^T) - diag(loss) (x) I with gain [Nr x Nr] row-major and loss [Nr];
 * the six bands vr_* [ndr x Nr], vt_* [ndt x Nvt], x_* [ndx x Nx] (init(), :1403-1470). */
int bte_fvm_create(int device, int Nr, int Nvt, int Nx, int ndr, int ndt, int ndx, const double* vr, const double* vt,
                   const double* w, const double* loss, const double* gain, const double* vr_l2r,
                   const double* vr_r2l, const double* vt_l2r, const double* vt_r2l, const double* x_l2r,
                   const double* x_r2l, bte_fvm** out);
int bte_fvm_destroy(bte_fvm* h);

/* The collision solve of the preconditioner, (I - c C)^-1 = diag(dinv) (x) I + H (x) 1 w^T
 * with c = gmres_pc_cv dt tau kappa: dinv [Nr] = 1 / (1 + c loss), H [Nr x Nr] row-major =
 * c D^-1 gain (D - c |w| gain)^-1, D = diag(1 + c loss). Replaces PmatC (:1346-1375). */
int bte_fvm_set_collision_inverse(bte_fvm* h, const double* dinv, const double* H);

/* Y = rhs_mvec(X) (:1915-1955): X v - dt tau (kappa C v + E (x) cA A_sign(E) v), the second
 * term zero at the inflow values, E [Nx]. Y must not alias X. */
int bte_fvm_mvec(bte_fvm* h, const bte_fvm_coef* c, const double* E, const double* X, double* Y, void* stream);

/* Y = step_op_split(E, X) with type XVTVRC (:1745-1870): the collision solve, then upwind
 * backward-Euler sweeps along v_r and v_theta at aE = cE E, and along x at ax v_r cos(theta)
 * after zeroing the inflow values, all with step hstep (= alpha dt). */
int bte_fvm_precond(bte_fvm* h, double cE, double ax, double hstep, const double* E, const double* X, double* Y,
                    void* stream);

/* One fully implicit step (:1890-2009): solves rhs_mvec(V') = V with its inflow values zeroed,
 * by restarted GMRES(restart) to ||r|| <= max(atol, rtol ||b||) or max_iter iterations;
 * V [Nr * Nvt * Nx] is replaced by V'. pc_mode: 0 the op-split step at alpha dt as a right
 * preconditioner (utils.py:1172-1262), 1 as a left one (utils.py:1266-1357), 2 none
 * (pc_type "none", :1979-1982; no collision inverse needed).
 * info4: iterations, ||r||, ||r|| / ||b||, status (0 converged, 1 not converged). */
int bte_fvm_step(bte_fvm* h, const bte_fvm_coef* c, double alpha, int pc_mode, const double* E, double* V, double rtol,
                 double atol, int restart, int max_iter, double* info4, void* stream);

/* The grids of the semi-Lagrangian step: x [Nx] ascending, the velocity domain [vmin, vmax]
 * of the cells (the basis's knot domain). */
int bte_fvm_set_sl_grid(bte_fvm* h, const double* x, double vmin, double vmax);

/* Y = step_adv_vx_sl(V) (:2244-2314): each value the trilinear interpolant of V, on the grid
 * padded by one layer in v_r and theta, at its departure point (x - dt ax v_r cos(theta) in x;
 * the velocity shifted by dt tau cA E along the field axis); zero outside the padded grid. */
int bte_fvm_sl_advect(bte_fvm* h, const bte_fvm_coef* c, const double* E, const double* V, double* Y, void* stream);

/* One semi-Lagrangian step (solver_type "sl_implicit", :2024-2027): the collision inverse of
 * bte_fvm_set_collision_inverse applied to step_adv_vx_sl(V). Y must not alias V. */
int bte_fvm_sl_step(bte_fvm* h, const bte_fvm_coef* c, const double* E, const double* V, double* Y, void* stream);

/* kernel launches issued by this handle so far */
long long bte_fvm_launches(const bte_fvm* h);
const char* bte_fvm_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
