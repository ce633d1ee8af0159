// Internal definition of a velocity-space grid handle: every operator the batched
// 0D3V steady-state / transient solves need, resident in device memory.
#pragma once
#include <vector>
#include <string>
#include <cuda_runtime.h>
#include "../../include/bte_gb300.h"

struct BteQuad {          // per-knot-interval Gauss-Legendre rule with its B-spline table
    int q = 0;            // points per non-degenerate knot interval
    int npts = 0;
    double* x = nullptr;  // [npts]
    double* w = nullptr;  // [npts]
    int* span = nullptr;  // [npts] knot span of each point (nonzero splines span-3..span)
    double* B = nullptr;  // [npts][3][4] values, first and second derivatives
};

struct BteGrid {
    // sizes
    int nsp = 0, lmax = 0, nsh = 0, n = 0, N = 0, ldj = 0;
    int nproc = 0, nspecies = 0, ee = 0, ntri = 0, nint = 0, spline_qpts = 5;
    double vth = 0, mw0 = 0, mByM = 0, ev_max = 0, Te = 0, c_adv = 0;
    double q0max = 0, advmax = 0, umax = 0, Mpmax = 0;
    int device = 0;

    // host copies
    std::vector<double> knots;
    std::vector<int> span_iv;            // knot span -> interval index (or -1)
    std::vector<int> proc_type, proc_species;
    std::vector<double> proc_threshold, proc_attach;
    std::vector<int> tri;                // ntri x 3 (q, l, s)
    std::vector<double> angA, angG;      // ntri x 2, ntri x 5

    // device: basis and quadrature
    double* d_t = nullptr;
    int* d_span_iv = nullptr;
    BteQuad q5, q10, q12;
    double* d_sig5 = nullptr;            // nproc x q5.npts, sigma at the collision rule
    int* d_sig_off = nullptr;            // nproc + 1 offsets into the tables
    double* d_sig_e = nullptr;
    double* d_sig_v = nullptr;
    int* d_proc_type = nullptr;
    int* d_proc_species = nullptr;
    double* d_proc_threshold = nullptr;
    double* d_proc_attach = nullptr;

    // device: radial operators (FP64). Band layout [p][dk + 3], dense layout row-major.
    double* d_Mr = nullptr;              // nsp x 7
    double* d_Minv = nullptr;            // nsp x nsp
    double* d_mm1 = nullptr;             // nsp x 7  int v^2 phi_p phi_k'
    double* d_mm2 = nullptr;             // nsp x 7  int v   phi_p phi_k
    double* d_q0 = nullptr;              // nspecies x nsp x nsp  (l = 0 block)
    double* d_q1 = nullptr;              // nspecies x nsp x 7    (l > 0 blocks)
    double* d_cgT = nullptr;             // nsp x 7               (l = 0 block)
    double* d_adv_coef = nullptr;        // nsh x 4: AM(q+1), AD(q+1), BM(q-1), BD(q-1)

    // device: functionals and constraint vectors (FP64)
    double* d_mass = nullptr;            // n
    double* d_temp = nullptr;            // n (scaled as the reference's _op_temp)
    double* d_mob = nullptr;             // nsp
    double* d_diff = nullptr;            // nsp
    double* d_rate = nullptr;            // nproc x nsp
    double* d_u = nullptr;               // n
    double* d_p = nullptr;               // n
    double* d_Mp = nullptr;              // n
    double* d_W = nullptr;               // nspecies x n
    double* d_invMd = nullptr;           // n, 1 / diag(M)
    double* d_vD = nullptr;              // n, D M p / |D M p| with D = diag(M)^-1

    // device: Coulomb (FP64)
    double* d_HL = nullptr;              // nsh x nsp x nsp
    double* d_GL = nullptr;              // nsh x nsp x nsp
    double* d_CA = nullptr;              // ntri x nsp x 7 x 7
    double* d_CB = nullptr;              // ntri x nsp x 7 x 7
    int* d_tri = nullptr;                // ntri x 3

    // device: FP32 copies for the mixed-precision Jacobian
    float* f_q0 = nullptr; float* f_q1 = nullptr; float* f_cgT = nullptr;
    float* f_mm1 = nullptr; float* f_mm2 = nullptr; float* f_Mr = nullptr;
    float* f_HL = nullptr; float* f_GL = nullptr; float* f_CA = nullptr; float* f_CB = nullptr;

    std::vector<void*> allocations;
    struct BteWork* work = nullptr;      // solver workspace, grown on demand
};

// assembly.cu
int bte_assemble(BteGrid* g, cudaStream_t s);
// newton.cu
struct BteWork;
BteWork* bte_work_get(BteGrid* g);
void bte_work_release(BteWork* w);
struct BteEngine;
int bte_engine_create_impl(BteGrid* g, int cap, int fcap, const bte_solve_opts* o, BteEngine** out);
void bte_engine_destroy_impl(BteEngine* e);
int bte_engine_admit_impl(BteEngine* e, int m, const double* n0, const double* ne, const double* ns_by_n0,
                          const double* Tg, const double* E, const double* f0, int want_ee, int32_t* slots_out,
                          cudaStream_t s);
int bte_engine_step_impl(BteEngine* e, int* n_done, int32_t* done_out, cudaStream_t s);
int bte_engine_collect_impl(BteEngine* e, int m, const int32_t* slots, double* f, int32_t* status, int32_t* iters,
                            cudaStream_t s);
int bte_engine_free_slots(const BteEngine* e);
int bte_engine_active(const BteEngine* e);
size_t bte_engine_bytes(const BteEngine* e);
int bte_engine_fp64_capacity(const BteEngine* e);
int bte_engine_capacity(const BteEngine* e);
BteGrid* bte_engine_grid(const BteEngine* e);
int bte_transient_impl(BteGrid* g, int P, const double* n0, const double* ne, const double* ns_by_n0,
                       const double* Tg, const double* E, const double* eRe, const double* eIm, double* f,
                       double* f_avg, int32_t* status, int32_t* iters, const bte_transient_opts* o, cudaStream_t s);
int bte_solve_impl(BteGrid* g, int P, const double* n0, const double* ne, const double* ns_by_n0,
                   const double* Tg, const double* E, double* f, int32_t* status, int32_t* iters,
                   const bte_solve_opts* opts, cudaStream_t s);
int bte_solve_info_impl(BteGrid* g, int P, double* r_final, double* r_initial, cudaStream_t s);
