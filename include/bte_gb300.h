/*
 * bte_gb300.h — C ABI of the GB300 (sm_103a) batched velocity-space Boltzmann library.
 *
 * Drop-in boundary for the hot path of Boltzsim (ut-padas/boltzmann), whose public
 * interface is the Python class `bte_0d3v_batched` (BESolver/python/bte_0d3v_batched.py).
 * Every entry point names the reference interface it replaces. Conventions:
 *   - plain pointers and sizes only; batch arrays are caller-owned DEVICE buffers
 *     unless the parameter says "host";
 *   - distributions are stored point-major: f[point * n + (p * num_sh + l)], with
 *     n = n_sp * (l_max + 1) and the reference's radial-major coefficient order
 *     (BESolver/python/spec_spherical.py:219-221);
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream);
 *   - every function returns 0 on success or a negative BTE_ERR_* code, and never
 *     exits the process; per-point solver outcomes go to an int32 status array.
 *   - one grid handle must not be used from two host threads at once.
 */
#ifndef BTE_GB300_H
#define BTE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct BteGrid bte_grid;

/* process kinds (reference: collisions.py:400-430, CollisionType EAR_G0..G3) */
#define BTE_PROC_ELASTIC 0
#define BTE_PROC_EXCITATION 1
#define BTE_PROC_IONIZATION 2
#define BTE_PROC_ATTACHMENT 3

/* arithmetic of the Newton linear solves */
#define BTE_PREC_FP64 0   /* plain: FP64 Jacobian, FP64 LU, FP64 residual            */
#define BTE_PREC_MIXED 1  /* FP32 Jacobian + FP32 LU, corrections against the FP64 residual */

typedef struct {
    int n_sp;                     /* number of cubic B-splines (reference argument Nr + 1)   */
    int l_max;                    /* spherical-harmonic modes l = 0..l_max, m = 0             */
    int spline_qpts;              /* Gauss points per knot interval, collision rule (5)      */
    int vspace_ext;               /* 0 = none, 1 = linear x1.2 (vspace_grid_extension)        */
    int ee;                       /* 1 = assemble the e-e Coulomb operators                   */
    double ev_max;                /* grid energy, eV                                         */
    double Te;                    /* normalisation temperature, eV (sets vth)                 */
    double mByM;                  /* m_e / M of the elastic process                           */
    int n_processes;
    int n_species;
    const int* proc_type;         /* host [n_processes] BTE_PROC_*                             */
    const int* proc_species;      /* host [n_processes] species index                          */
    const double* proc_threshold; /* host [n_processes] eV (ignored for elastic)               */
    const double* proc_attach;    /* host [n_processes] attachment energy, eV                  */
    const int* sigma_offsets;     /* host [n_processes + 1] offsets into the two tables below  */
    const double* sigma_energy;   /* host, eV, increasing per process                          */
    const double* sigma_values;   /* host, m^2                                                 */
    int device;                   /* CUDA device ordinal                                       */
    int plain_knots;              /* 0: knots snapped to the process thresholds (the 0D3V
                                     solver, basis.py:356-362); 1: uniform knots only (the 1D3V
                                     solver's basis, bte_1d3v_solver.py:356, sig_pts=None)    */
} bte_grid_desc;

typedef struct {
    double atol, rtol;            /* stop when ||r|| <= atol + rtol * ||r0|| (per point)       */
    int max_iter;
    double alpha_min, alpha_rho, line_search_c;  /* Armijo backtracking                       */
    int ee;                       /* include the e-e Coulomb term                              */
    int precision;                /* BTE_PREC_FP64 or BTE_PREC_MIXED                           */
    int refine;                   /* mixed form: at most this many FP64 refinement passes per
                                     Newton step (0-8); a point stops once its correction
                                     contracts 4x, and goes to the FP64 path if it does not
                                     contract at all                                          */
    int krylov;                   /* mixed form: GMRES on the FP32 factors for a point whose
                                     refinement does not contract, before it goes to the FP64
                                     path. 0: for bordered sizes n + 1 > 512 (default);
                                     1: for every size; 2: for every point of every Newton
                                     step (diagnostics); -1: never. No counterpart in the
                                     reference, which inverts in FP64                         */
    int lu_kernel;                /* mixed form: FP32 factorization of the Newton systems.
                                     0: the library's choice; 2: split-TF32 trailing updates
                                     on the tensor cores (bordered sizes n + 1 <= 512), two
                                     CTAs per SM; 4: the same with one CTA per SM; 5: with
                                     128 threads per CTA; 3: SIMT
                                     left-looking (n + 1 <= 512); 1: SIMT right-looking.
                                     Sizes a kernel does not take fall back to the library's
                                     choice                                                   */
    int lu64_kernel;              /* FP64 factorizations (the plain form, and the mixed form's
                                     FP64 lane): 0: the library's choice (6); 1: one CTA per
                                     system; 6: each system split over many CTAs            */
    int reserved[2];
} bte_solve_opts;

/* Options of the transient solve (the reference's args.dt / cycles / Efreq). */
typedef struct {
    double atol, rtol;   /* per point: ||r|| <= atol or ||r|| <= rtol ||r_0|| ends a step's chord iteration */
    int max_iter;        /* chord iterations per step */
    int ee;              /* include e-e collisions (grid must have them) */
    int precision;       /* BTE_PREC_FP64 or BTE_PREC_MIXED; the step Jacobian M - dt tau dF/dh is
                            factored in FP64 in both (it carries the mass matrix's conditioning,
                            beyond FP32 factors) */
    double dt;           /* time step in RF periods */
    double cycles;       /* simulated time in RF periods */
    double efreq;        /* field frequency in Hz; 0: constant field E and tau = 1e-7 s */
    int reserved[6];
} bte_transient_opts;

/* Build a grid and assemble every operator on the device (FP64).
 * Replaces bte_0d3v_batched.__init__ + assemble_operators
 * (BESolver/python/bte_0d3v_batched.py:138-306, 310-479). */
int bte_grid_create(const bte_grid_desc* desc, bte_grid** out, void* stream);

/* Release a grid and all its device memory. */
int bte_grid_destroy(bte_grid* g);

/* Sizes and scalars of a grid: ints = {n_sp, l_max, num_sh, n, n_intervals, n_triples,
 * n_processes, n_species}, dbls = {vth, maxwellian(0), v_max/vth, mByM}.
 * Replaces the attributes _par_vth / _op_spec_sp read by callers (bte_0d3v_batched.py:155-160). */
int bte_grid_info(const bte_grid* g, int* ints8, double* dbls4);

/* Copy one assembled operator, expanded to the reference's dense layout, into the
 * caller's device buffer `out` of `count` doubles. `which`: see BTE_OP_*.
 * Replaces reading _op_mass_mat, _op_advection, _op_col_en, ... (bte_0d3v_batched.py:359-476). */
#define BTE_OP_KNOTS 0      /* n_sp + 4                                              */
#define BTE_OP_MASS 1       /* n x n        spec_spherical.compute_mass_matrix       */
#define BTE_OP_MINV 2       /* n x n        spec_spherical.inverse_mass_mat          */
#define BTE_OP_ADV_RAW 3    /* n x n        compute_advection_matix (unscaled)       */
#define BTE_OP_COL_RAW 4    /* n_species x n x n  sum of assemble_mat per species     */
#define BTE_OP_COL_GT_RAW 5 /* n x n        electron_gas_temperature                 */
#define BTE_OP_MASS_VEC 6   /* n            utils.mass_op                            */
#define BTE_OP_TEMP_VEC 7   /* n            utils.temp_op * 0.5 m_e (2/3/k_B) / K_1eV */
#define BTE_OP_MOBILITY 8   /* n_sp         utils.mobility_op                        */
#define BTE_OP_DIFFUSION 9  /* n_sp         utils.diffusion_op                       */
#define BTE_OP_RATES 10     /* n_proc x n_sp utils.reaction_rates_op per process     */
#define BTE_OP_HL 11        /* n x n        compute_rosenbluth_potentials_op (hl)    */
#define BTE_OP_GL 12        /* n x n        compute_rosenbluth_potentials_op (gl)    */
#define BTE_OP_CC_A 13      /* n x n x n    coulomb_collision_op_assembly (cc_a)     */
#define BTE_OP_CC_B 14      /* n x n x n    coulomb_collision_op_assembly (cc_b)     */
#define BTE_OP_RADIAL_V3 15 /* n_sp x n_sp  int v^3 phi_p phi_k dv: the 1D3V x-advection radial
                                   integral (bte_1d3v_solver.py:529-564, compute_spatial_advection_op) */
int bte_grid_export(const bte_grid* g, int which, double* out, size_t count, void* stream);

/* Maxwellian initial state for P points (device f, P x n).
 * Replaces bte_0d3v_batched.initialize(grid, n_pts, "maxwellian") (bte_0d3v_batched.py:481-520). */
int bte_initialize(const bte_grid* g, int P, double* f, void* stream);

/* The Maxwellian initial state of bte_initialize (equal to round-off), from a call that
 * allocates no device memory. It is meant for callers that cannot allocate at the point where
 * they initialize points: a serving process whose device memory is all reserved by another
 * allocator (a caching allocator that holds the whole pool, or a job at its memory cap),
 * where a stream-ordered allocation can fail with out-of-memory or stall while the pool
 * grows. The call's scratch (the radial projection, n_sp doubles, and the angular factors,
 * num_sh doubles) lives in one static device array of the library, 4,160 bytes, which every
 * GPU that loads the library holds until the process exits; grids with
 * n_sp > BTE_INIT_NOALLOC_MAX_NSP or num_sh > BTE_INIT_NOALLOC_MAX_SH are rejected with
 * BTE_ERR_ARG and a message naming the limit. The caller passes f as for bte_initialize.
 * The first call on each device looks up the scratch's device address (this can load the
 * library's device code), so make that first call during set-up, before any stream capture.
 * All calls on a device share the one scratch array: calls that overlap on the GPU (other
 * streams, other host threads) race on it, so the caller serialises them. Every element
 * read is written earlier in the same call, so nothing in the scratch needs to start at
 * zero. Synchronizes `stream` before returning, as bte_initialize does.
 * No counterpart in the reference: an addition of this library. */
#define BTE_INIT_NOALLOC_MAX_NSP 512
#define BTE_INIT_NOALLOC_MAX_SH 8
int bte_initialize_noalloc(const bte_grid* g, int P, double* f, void* stream);

/* Steady-state solve of P independent points. Device inputs n0, ne, Tg, E [P],
 * ns_by_n0 [n_species x P]; f [P x n] in: initial state (any positive multiple),
 * out: the normalized distribution (normalized_distribution). status/iters [P] int32.
 * Replaces bte_0d3v_batched.solve(..., "steady-state") / steady_state_solve
 * (bte_0d3v_batched.py:882-979, 1034-1047). */
int bte_solve_steady(bte_grid* g, int P, const double* n0, const double* ne, const double* ns_by_n0,
                     const double* Tg, const double* E, double* f, int32_t* status, int32_t* iters,
                     const bte_solve_opts* opts, void* stream);

/* Per-point merit norms ||Q^T M^-1 F|| of the last bte_solve_steady on this grid (device
 * buffers [P]): at the returned state and at the initial state. Replaces the residual
 * printout of steady_state_solve (bte_0d3v_batched.py:960-963, 970-971). */
/* Transient solve of P points: backward Euler over `cycles` RF periods in steps of dt
 * (t in periods, tau = 1 / efreq), E(t) = eRe cos 2 pi t + eIm sin 2 pi t when efreq > 0,
 * else the constant E; each step by a chord Newton iteration on the mass-conserving
 * increment with the Jacobian frozen at the step's start. f [P x n] in: initial state;
 * out: the final state (mass-normalized, as the reference returns u). f_avg [P x n] (may be
 * NULL): normalized distribution of the last completed cycle average, for bte_qoi with
 * effective_mobility = 0. status [P] 0, or BTE_ST_MAXITER if a step did not converge (the
 * call then returns BTE_ERR_STATE); iters [P] total chord iterations.
 * Replaces bte_0d3v_batched.solve(..., "transient") (bte_0d3v_batched.py:1063-1155) with
 * newton_solver_batched (:59-126). */
int bte_solve_transient(bte_grid* g, int P, const double* n0, const double* ne, const double* ns_by_n0,
                        const double* Tg, const double* E, const double* eRe, const double* eIm, double* f,
                        double* f_avg, int32_t* status, int32_t* iters, const bte_transient_opts* opts, void* stream);

int bte_solve_info(bte_grid* g, int P, double* r_final, double* r_initial, void* stream);

/* Quantities of interest of P normalized distributions (device f [P x n]); outputs
 * [P] each and rates [n_proc x P]. effective_mobility as in the reference.
 * Replaces bte_0d3v_batched.compute_QoIs (bte_0d3v_batched.py:1163-1202). */
int bte_qoi(const bte_grid* g, int P, const double* f, const double* n0, const double* E,
            int effective_mobility, double* energy, double* mobility, double* diffusion,
            double* rates, void* stream);

/* Batched dense LU with partial pivoting, in place, on P ROW-major N x N matrices
 * (A[r * ld + c], N <= 2048) with matrix stride `stride` (elements). dtype 0 = FP64, 1 = FP32.
 * Rows are not exchanged in memory: piv [P x N] int32 receives the permutation, and row
 * perm[r] of the output holds row r of L\U (L unit lower). info [P] = 0 or the 1-based
 * pivot position of the first zero pivot.
 * Replaces the xp.linalg.inv call of bte_0d3v_batched.batched_inv (bte_0d3v_batched.py:856-880). */
int bte_lu_factor(int dtype, int P, int N, void* A, int ld, long long stride, int32_t* piv, int32_t* info,
                  void* stream);

/* As bte_lu_factor with an explicit kernel: 0 = automatic (FP32: tensor-core kernel for
 * N <= 512, right-looking above; FP64: right-looking),
 * 1 = right-looking for every N, 2 = FP32 only, N <= 512: trailing updates on the tcgen05
 * tensor cores in split TF32 (FP32-accurate factors), 3 = left-looking (N <= 512),
 * 4 = as 2 with one CTA per SM instead of two (fewer matrices in flight, kept in L2),
 * 5 = as 2 with 128 threads per CTA (less pivot-search work per matrix),
 * 6 = FP64 only: each factorization split over many CTAs (per panel: pivoting, triangular
 *     solve, 64 x 64 trailing tiles as separate launches), for few large FP64 systems.
 * No counterpart in the reference; used to cross-check the factorizations. */
int bte_lu_factor_ex(int dtype, int P, int N, void* A, int ld, long long stride, int32_t* piv, int32_t* info,
                     int kernel, void* stream);

/* Solve A x = b for one right-hand side per matrix using bte_lu_factor's output;
 * b [P x N] (contiguous per point) is overwritten by x. Same dtype as the factors. */
int bte_lu_solve(int dtype, int P, int N, const void* A, int ld, long long stride,
                 const int32_t* piv, void* b, void* stream);

/* Radial components f_l(eps) of P distributions (device f [P x n]) at n_ev energies
 * (device ev, eV): out [P x num_sh x n_ev], out[pt][l][e] = sum_p f[pt][p, l] B_p(v(eps_e)).
 * Replaces bte_0d3v_batched.compute_radial_components (bte_0d3v_batched.py:1219-1239). */
int bte_radial_components(const bte_grid* g, int P, const double* f, int n_ev, const double* ev, double* out,
                          void* stream);

/* Reset the library's kernel-launch counter and per-family statistics; enable_timing = 1
 * also brackets every solver launch with CUDA events (small overhead).
 * Replaces bte_0d3v_batched.profile_reset (bte_0d3v_batched.py:1241-1246). */
int bte_stats_reset(int enable_timing);

/* Statistics since the last reset: out[0] = kernel launches; then per family
 * {residual, jacobian, lu_factor (FP32), lu_solve, refine, other, lu_factor_fp64}: launches,
 * device ms, algorithmic flops, algorithmic bytes; out[29] = points of the mixed form handed
 * to the FP64 path (count >= 30 doubles); out[30..34] = their reasons {max_iter, line
 * search, non-finite, singular, refinement} when count >= 35.
 * Replaces bte_0d3v_batched.profile_stats (bte_0d3v_batched.py:1248-1315). */
int bte_stats(double* out, int count);

/* ---- Serving engine: continuous batching of steady-state solves on one grid ----
 * The reference has no serving loop; this is the device side of the request loop in
 * boltzmann_gb300/serving.py. An engine owns `capacity` point slots on one grid (state,
 * Jacobian buffers and parameters resident on the device). Points are admitted into free
 * slots between Newton iterations and retire when their own solve ends, so requests that
 * arrive while others run share the same kernel launches. Each admitted point runs the
 * reference driver's solve sequence (bte_0d3v_batched_driver.py:192-204): a steady solve
 * without e-e collisions from its initial state, then, if `ee` was set at admission, one
 * with them from that result; per point the arithmetic is that of two bte_solve_steady
 * calls. In the mixed form a point whose FP32 solve fails continues in an FP64 lane of
 * `fp64_capacity` slots. One engine is driven by one host thread on one stream at a time;
 * engines of different grids may run concurrently on different streams. */
typedef struct BteEngine bte_engine;
int bte_engine_create(bte_grid* g, int capacity, int fp64_capacity, const bte_solve_opts* opts, bte_engine** out);
int bte_engine_destroy(bte_engine* e);
/* Admit P points (device arrays: n0, ne, Tg, E [P]; ns_by_n0 [n_species x P]; f0 [P x n],
 * any positive multiple of the initial state). Fails with BTE_ERR_STATE if fewer than P slots
 * are free. slots (host, P) receives the slot of each point. */
int bte_engine_admit(bte_engine* e, int P, const double* n0, const double* ne, const double* ns_by_n0,
                     const double* Tg, const double* E, const double* f0, int ee, int32_t* slots, void* stream);
/* One Newton iteration of every running point. n_done (host) receives the number of points
 * whose solve ended in this step and done_slots (host, capacity) their slots. */
int bte_engine_step(bte_engine* e, int* n_done, int32_t* done_slots, void* stream);
/* Results of P finished slots (host list): f [P x n] the normalized distribution
 * (normalized_distribution, bte_0d3v_batched.py:1204-1217), status and iters (device int32,
 * may be NULL: total Newton iterations of both solves). The slots become free. */
int bte_engine_collect(bte_engine* e, int P, const int32_t* slots, double* f, int32_t* status, int32_t* iters,
                       void* stream);
/* ints4 = {capacity, free slots, running points, fp64 capacity}; bytes = device memory the
 * engine holds (its per-slot footprint is bytes / capacity). */
int bte_engine_info(const bte_engine* e, int* ints4, size_t* bytes);

/* Last CUDA error string seen by the library on this thread (never NULL). */
const char* bte_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* BTE_GB300_H */
