// C ABI of the batched velocity-space library (declarations in include/bte_gb300.h).
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <algorithm>
#include <mutex>
#include "bte_common.cuh"
#include "bte_grid.h"

template <typename T>
cudaError_t bte_lu_factor_t(int P, int N, int NC, T* A, int ld, long long stride, int32_t* piv, int32_t* info,
                            cudaStream_t s, int kernel);
template <typename T>
cudaError_t bte_lu_solve_t(int P, int N, const T* A, int ld, long long stride, const int32_t* piv, T* b, int mode,
                           cudaStream_t s, const int32_t* mats = nullptr);
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w);

static thread_local std::string g_last_error = "";

static int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
static int cuda_fail(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return BTE_ERR_CUDA;
}
#define CUDA_OR_FAIL(x, where) do { cudaError_t _e = (x); if (_e != cudaSuccess) return cuda_fail(_e, where); } while (0)

static void grid_free(BteGrid* g) {
    if (!g) return;
    if (g->work) { bte_work_release(g->work); g->work = nullptr; }
    for (void* p : g->allocations) cudaFree(p);
    g->allocations.clear();
    delete g;
}

// Knot vector of bte_0d3v_batched.assemble_operators (bte_0d3v_batched.py:334-351) with
// BSpline.uniform_knots (basis.py:640-653) and threshold snapping (basis.py:356-362).
static std::vector<double> make_knots(int nsp, double k0, double k1, const std::vector<double>& sig) {
    const int p = BTE_SP_ORDER;
    std::vector<double> t;
    for (int i = 0; i < p; ++i) t.push_back(k0);
    const int num = nsp - p;
    const double step = (k1 - k0) / num;  // numpy.linspace(endpoint=False): i * step + start
    for (int i = 0; i < num; ++i) t.push_back(i * step + k0);
    for (int i = 0; i < p + 1; ++i) t.push_back(k1);
    return t;
}

static void snap_knots(std::vector<double>& t, double d0, double d1, const std::vector<double>& sig) {
    const int p = BTE_SP_ORDER;
    for (double s : sig) {
        if (!(s > d0 && s < d1)) continue;
        int idx = 0;
        double best = std::fabs(t[0] - s);
        for (int i = 1; i < (int)t.size(); ++i) {
            double d = std::fabs(t[i] - s);
            if (d < best) { best = d; idx = i; }
        }
        if (idx > p + 1 && idx < (int)t.size() - p - 1) t[idx] = s;
    }
}

extern "C" {

const char* bte_last_error(void) { return g_last_error.c_str(); }

int bte_grid_create(const bte_grid_desc* d, bte_grid** out, void* stream) {
    if (!d || !out) return fail(BTE_ERR_ARG, "null argument");
    *out = nullptr;
    if (d->n_sp < 8 || d->n_sp > 4096) return fail(BTE_ERR_ARG, "n_sp out of range [8, 4096]");
    if (d->l_max < 0 || d->l_max > 4) return fail(BTE_ERR_ARG, "l_max out of range [0, 4]");
    if (d->spline_qpts < 1 || d->spline_qpts > 16) return fail(BTE_ERR_ARG, "spline_qpts out of range [1, 16]");
    if (d->n_processes < 1 || d->n_species < 1) return fail(BTE_ERR_ARG, "need at least one process and species");
    if (!(d->ev_max > 0) || !(d->Te > 0)) return fail(BTE_ERR_ARG, "ev_max and Te must be positive");
    if (d->vspace_ext != 0 && d->vspace_ext != 1) return fail(BTE_ERR_ARG, "vspace_ext must be 0 (none) or 1 (linear)");
    if (d->plain_knots != 0 && d->plain_knots != 1) return fail(BTE_ERR_ARG, "plain_knots must be 0 or 1");
    for (int i = 0; i < d->n_processes; ++i) {
        if (d->proc_type[i] < 0 || d->proc_type[i] > 3) return fail(BTE_ERR_ARG, "unknown process type");
        if (d->proc_species[i] < 0 || d->proc_species[i] >= d->n_species) return fail(BTE_ERR_ARG, "bad species index");
        int m = d->sigma_offsets[i + 1] - d->sigma_offsets[i];
        if (m < 2) return fail(BTE_ERR_ARG, "cross-section table needs at least 2 points");
    }
    CUDA_OR_FAIL(cudaSetDevice(d->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    BteGrid* g = new BteGrid();
    g->device = d->device;
    g->nsp = d->n_sp;
    g->lmax = d->l_max;
    g->nsh = d->l_max + 1;
    g->n = g->nsp * g->nsh;
    g->N = g->n + 1;
    g->nproc = d->n_processes;
    g->nspecies = d->n_species;
    g->ee = d->ee;
    g->spline_qpts = d->spline_qpts;
    g->mByM = d->mByM;
    g->ev_max = d->ev_max;
    g->Te = d->Te;
    const double kB = BTE_KB, me = BTE_ME, ev = BTE_QE;
    const double T = d->Te * (ev / kB);
    g->vth = std::sqrt(2.0 * kB * T / me);                       // collisions.py:20-25
    const double cg = std::sqrt(2.0 * (BTE_QE / BTE_ME));      // bte_0d3v_batched.py:163
    g->mw0 = 1.0 / std::pow(g->vth * std::sqrt(M_PI), 3.0);    // utils.py:713-715 at 0
    g->c_adv = (1.0 / g->vth) * (BTE_QE / BTE_ME);
    std::vector<double> sig;
    for (int i = 0; i < g->nproc; ++i) {
        g->proc_type.push_back(d->proc_type[i]);
        g->proc_species.push_back(d->proc_species[i]);
        g->proc_threshold.push_back(d->proc_threshold[i]);
        g->proc_attach.push_back(d->proc_attach[i]);
        if (d->proc_type[i] != BTE_PROC_ELASTIC && d->proc_threshold[i] > 0) sig.push_back(d->proc_threshold[i]);
    }
    std::sort(sig.begin(), sig.end());
    sig.erase(std::unique(sig.begin(), sig.end()), sig.end());
    std::vector<double> dg;
    for (double sv : sig) dg.push_back(std::sqrt(sv) * cg / g->vth);
    const double k0 = std::sqrt(0.0) * cg / g->vth, k1 = std::sqrt(d->ev_max) * cg / g->vth;
    g->knots = make_knots(g->nsp, k0, d->vspace_ext == 1 ? 1.2 * k1 : k1, dg);
    if (!d->plain_knots) snap_knots(g->knots, k0, k1, dg);
    for (size_t j = 0; j + 1 < g->knots.size(); ++j) {
        if (g->knots[j] != g->knots[j + 1]) g->span_iv.push_back(g->nint++);
        else g->span_iv.push_back(-1);
    }
    // cross-section tables
    int tot = d->sigma_offsets[g->nproc];
    auto up = [&](void** p, const void* src, size_t bytes) -> bool {
        if (cudaMalloc(p, std::max<size_t>(bytes, 8)) != cudaSuccess) return false;
        g->allocations.push_back(*p);
        return cudaMemcpyAsync(*p, src, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
    };
    bool ok = up((void**)&g->d_sig_off, d->sigma_offsets, (g->nproc + 1) * sizeof(int)) &&
              up((void**)&g->d_sig_e, d->sigma_energy, tot * sizeof(double)) &&
              up((void**)&g->d_sig_v, d->sigma_values, tot * sizeof(double));
    if (!ok) { grid_free(g); return fail(BTE_ERR_ALLOC, "device allocation failed"); }
    int rc = bte_assemble(g, s);
    if (rc != BTE_OK) {
        cudaError_t e = cudaGetLastError();
        grid_free(g);
        return fail(rc, std::string("assembly failed: ") + cudaGetErrorString(e));
    }
    *out = g;
    return BTE_OK;
}

int bte_grid_destroy(bte_grid* g) {
    if (!g) return fail(BTE_ERR_ARG, "null grid");
    cudaSetDevice(g->device);
    cudaDeviceSynchronize();
    grid_free(g);
    return BTE_OK;
}

int bte_grid_info(const bte_grid* g, int* ints, double* dbls) {
    if (!g || !ints || !dbls) return fail(BTE_ERR_ARG, "null argument");
    ints[0] = g->nsp; ints[1] = g->lmax; ints[2] = g->nsh; ints[3] = g->n;
    ints[4] = g->nint; ints[5] = g->ntri; ints[6] = g->nproc; ints[7] = g->nspecies;
    dbls[0] = g->vth; dbls[1] = g->mw0; dbls[2] = g->knots.back(); dbls[3] = g->mByM;
    return BTE_OK;
}

}  // extern "C"

__global__ void k_radial(int nsp, int nsh, const double* __restrict__ t, double scale, const double* __restrict__ f,
                         int n_ev, const double* __restrict__ ev, double* out, int P) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    int pt = blockIdx.y;
    if (e >= n_ev || pt >= P) return;
    double v = sqrt(ev[e]) * scale;
    double d[3][4];
    int s = bspline_eval(t, nsp, v, 0, d);
    const int n = nsp * nsh;
    for (int l = 0; l < nsh; ++l) {
        double acc = 0.0;
        if (s >= 0)
            for (int j = 0; j < 4; ++j) acc += f[(size_t)pt * n + (s - BTE_SP_ORDER + j) * nsh + l] * d[0][j];
        out[((size_t)pt * nsh + l) * n_ev + e] = acc;
    }
}

extern "C" int bte_radial_components(const bte_grid* g, int P, const double* f, int n_ev, const double* ev,
                                     double* out, void* stream) {
    if (!g || P < 0 || n_ev < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P == 0 || n_ev == 0) return BTE_OK;
    if (!f || !ev || !out) return fail(BTE_ERR_ARG, "null buffer");
    cudaSetDevice(g->device);
    const double cg = std::sqrt(2.0 * (BTE_QE / BTE_ME));
    dim3 gr((n_ev + 127) / 128, P);
    k_radial<<<gr, 128, 0, (cudaStream_t)stream>>>(g->nsp, g->nsh, g->d_t, cg / g->vth, f, n_ev, ev, out, P);
    CUDA_OR_FAIL(cudaGetLastError(), "k_radial");
    return BTE_OK;
}

// ---------------------------------------------------------------------------------
// dense expansions for export
// ---------------------------------------------------------------------------------
struct ExportView {
    int nsp, nsh, n, lmax, nspecies, nproc, ntri;
    const double *t, *Mr, *Minv, *mm1, *mm2, *q0, *q1, *cgT, *adv_coef, *mass, *temp, *mob, *diff, *rate, *HL, *GL,
        *CA, *CB;
    const int* tri;
};

__global__ void k_export(ExportView v, int which, double* out, size_t count) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int n = v.n, nsh = v.nsh, nsp = v.nsp;
    double val = 0.0;
    switch (which) {
        case BTE_OP_KNOTS: val = v.t[i]; break;
        case BTE_OP_MASS_VEC: val = v.mass[i]; break;
        case BTE_OP_TEMP_VEC: val = v.temp[i]; break;
        case BTE_OP_MOBILITY: val = v.mob[i]; break;
        case BTE_OP_DIFFUSION: val = v.diff[i]; break;
        case BTE_OP_RATES: val = v.rate[i]; break;
        case BTE_OP_CC_A:
        case BTE_OP_CC_B: {
            size_t a = i / ((size_t)n * n), rem = i % ((size_t)n * n);
            int b = (int)(rem / n), c = (int)(rem % n);
            int p = (int)a / nsh, q = (int)a % nsh, k = b / nsh, l = b % nsh, r = c / nsh, s = c % nsh;
            int dk = k - p, dr = r - p;
            if (abs(dk) <= BTE_BAND && abs(dr) <= BTE_BAND) {
                for (int t = 0; t < v.ntri; ++t)
                    if (v.tri[3 * t] == q && v.tri[3 * t + 1] == l && v.tri[3 * t + 2] == s) {
                        const double* C = (which == BTE_OP_CC_A) ? v.CA : v.CB;
                        val = C[(((size_t)t * nsp + p) * BTE_NB + dk + BTE_BAND) * BTE_NB + dr + BTE_BAND];
                    }
            }
            break;
        }
        default: {
            size_t sp = i / ((size_t)n * n), rem = i % ((size_t)n * n);
            int a = (int)(rem / n), b = (int)(rem % n);
            int p = a / nsh, q = a % nsh, k = b / nsh, l = b % nsh, dk = k - p;
            bool band = abs(dk) <= BTE_BAND;
            int bi = p * BTE_NB + dk + BTE_BAND;
            if (which == BTE_OP_MASS) { if (q == l && band) val = v.Mr[bi]; }
            else if (which == BTE_OP_MINV) { if (q == l) val = v.Minv[(size_t)p * nsp + k]; }
            else if (which == BTE_OP_ADV_RAW) {
                if (band && l == q + 1) val = v.mm1[bi] * v.adv_coef[q * 4 + 0] + v.adv_coef[q * 4 + 1] * v.mm2[bi];
                if (band && l == q - 1) val = v.mm1[bi] * v.adv_coef[q * 4 + 2] + v.adv_coef[q * 4 + 3] * v.mm2[bi];
            } else if (which == BTE_OP_COL_RAW) {
                if (q == l) {
                    if (q == 0) val = v.q0[((size_t)sp * nsp + p) * nsp + k];
                    else if (band) val = v.q1[((size_t)sp * nsp + p) * BTE_NB + dk + BTE_BAND];
                }
            } else if (which == BTE_OP_COL_GT_RAW) { if (q == 0 && l == 0 && band) val = v.cgT[bi]; }
            else if (which == BTE_OP_HL || which == BTE_OP_GL) {
                const double* H = (which == BTE_OP_HL) ? v.HL : v.GL;
                if (q == l && H) val = H[((size_t)q * nsp + p) * nsp + k];
            }
            break;
        }
    }
    out[i] = val;
}

// Maxwellian projection (bte_0d3v_batched.py:481-520 via utils.function_to_basis, utils.py:475-532)
// int v^3 phi_p phi_k dv over the whole radial domain (the 1D3V spatial-advection radial
// integral, bte_1d3v_solver.py:529-564): per-interval Gauss-Legendre, exact for the degree-9
// integrand; one thread per (p, k), zero outside |p - k| <= 3
__global__ void k_radial_v3(int nsp, const int* __restrict__ iv_span, int q, const double* __restrict__ x,
                            const double* __restrict__ w, const int* __restrict__ span, const double* __restrict__ B,
                            double* out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nsp * nsp) return;
    const int p = e / nsp, k = e % nsp;
    double s = 0.0;
    if (abs(p - k) <= BTE_SP_ORDER) {
        // the supports of p and k overlap on knot spans max(p,k) .. min(p,k) + 3
        for (int j = max(p, k); j <= min(p, k) + BTE_SP_ORDER; ++j) {
            const int iv = iv_span[j];
            if (iv < 0) continue;
            for (int gq = 0; gq < q; ++gq) {
                const int idx = iv * q + gq;
                const int jp = p - (span[idx] - BTE_SP_ORDER), jk = k - (span[idx] - BTE_SP_ORDER);
                if (jp < 0 || jp > 3 || jk < 0 || jk > 3) continue;
                const double xx = x[idx];
                s += w[idx] * xx * xx * xx * B[(idx * 3) * 4 + jp] * B[(idx * 3) * 4 + jk];
            }
        }
    }
    out[e] = s;
}

__global__ void k_maxwell_rhs(int nsp, const int* __restrict__ iv_span, int q, const double* __restrict__ x,
                              const double* __restrict__ w, const int* __restrict__ span, const double* __restrict__ B,
                              double* radial) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nsp) return;
    const double c = 1.0 / pow(sqrt(BTE_PI), 3.0);
    double s = 0.0;
    for (int j = p; j <= p + BTE_SP_ORDER; ++j) {
        int iv = iv_span[j];
        if (iv < 0) continue;
        for (int g = 0; g < q; ++g) {
            int idx = iv * q + g;
            int jj = p - (span[idx] - BTE_SP_ORDER);
            double bp = (jj >= 0 && jj <= 3) ? B[(idx * 3) * 4 + jj] : 0.0;
            double xx = x[idx];
            s += w[idx] * (c * exp(-(xx * xx)) * xx * xx) * bp;
        }
    }
    radial[p] = s;
}

__global__ void k_maxwell_fill(int nsp, int nsh, const double* __restrict__ Minv, const double* __restrict__ radial,
                               const double* __restrict__ ang, double* f, int P) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    int n = nsp * nsh;
    if (a >= n) return;
    int p = a / nsh, l = a % nsh;
    double s = 0.0;
    for (int c = 0; c < nsp; ++c) s += Minv[(size_t)p * nsp + c] * radial[c];
    s *= ang[l];
    for (int pt = 0; pt < P; ++pt) f[(size_t)pt * n + a] = s;
}

// compute_QoIs (bte_0d3v_batched.py:1163-1202), one thread per point
__global__ void k_qoi(int nsp, int nsh, int nproc, double mw0, double vth, const double* __restrict__ mass,
                      const double* __restrict__ temp, const double* __restrict__ mob, const double* __restrict__ diff,
                      const double* __restrict__ rate, const double* __restrict__ f, const double* __restrict__ n0,
                      const double* __restrict__ E, int eff, double* energy, double* mobility, double* diffusion,
                      double* rates, int P) {
    int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= P) return;
    const int n = nsp * nsh;
    const double* ff = f + (size_t)pt * n;
    const double cg = sqrt(2.0 * (BTE_QE / BTE_ME));
    double mm = 0.0, tt = 0.0;
    for (int i = 0; i < n; ++i) { mm += mass[i] * ff[i]; tt += temp[i] * ff[i]; }
    mm = mm * mw0 * (vth * vth * vth);
    energy[pt] = 1.5 * tt * mw0 * pow(vth, 5.0) / mm;
    double m1 = 0.0, d0 = 0.0;
    for (int p = 0; p < nsp; ++p) {
        if (nsh > 1) m1 += mob[p] * (sqrt(3.0) * ff[p * nsh + 1]);
        d0 += diff[p] * ff[p * nsh];
    }
    double fac = eff ? (-(cg / (3.0 * (E[pt] / n0[pt])))) : (-(cg / (3.0 * (1.0 / n0[pt]))));
    mobility[pt] = m1 * fac;
    diffusion[pt] = d0 * (cg / 3.0);
    for (int g = 0; g < nproc; ++g) {
        double r = 0.0;
        for (int p = 0; p < nsp; ++p) r += rate[(size_t)g * nsp + p] * ff[p * nsh];
        rates[(size_t)g * P + pt] = r;
    }
}

extern "C" {

int bte_grid_export(const bte_grid* g, int which, double* out, size_t count, void* stream) {
    if (!g || !out) return fail(BTE_ERR_ARG, "null argument");
    const size_t n = g->n, nsp = g->nsp;
    size_t need = 0;
    switch (which) {
        case BTE_OP_KNOTS: need = g->knots.size(); break;
        case BTE_OP_MASS: case BTE_OP_MINV: case BTE_OP_ADV_RAW: case BTE_OP_COL_GT_RAW: need = n * n; break;
        case BTE_OP_HL: case BTE_OP_GL: if (!g->ee) return fail(BTE_ERR_STATE, "grid built without e-e"); need = n * n; break;
        case BTE_OP_COL_RAW: need = (size_t)g->nspecies * n * n; break;
        case BTE_OP_RADIAL_V3: need = nsp * nsp; break;
        case BTE_OP_MASS_VEC: case BTE_OP_TEMP_VEC: need = n; break;
        case BTE_OP_MOBILITY: case BTE_OP_DIFFUSION: need = nsp; break;
        case BTE_OP_RATES: need = (size_t)g->nproc * nsp; break;
        case BTE_OP_CC_A: case BTE_OP_CC_B:
            if (!g->ee) return fail(BTE_ERR_STATE, "grid built without e-e");
            need = n * n * n; break;
        default: return fail(BTE_ERR_ARG, "unknown operator id");
    }
    if (count != need) return fail(BTE_ERR_ARG, "count does not match the operator size");
    cudaSetDevice(g->device);
    if (which == BTE_OP_RADIAL_V3) {
        k_radial_v3<<<(unsigned)((need + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
            g->nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span, g->q5.B, out);
        CUDA_OR_FAIL(cudaGetLastError(), "k_radial_v3");
        return BTE_OK;
    }
    ExportView v{g->nsp, g->nsh, g->n, g->lmax, g->nspecies, g->nproc, g->ntri, g->d_t, g->d_Mr, g->d_Minv, g->d_mm1,
                 g->d_mm2, g->d_q0, g->d_q1, g->d_cgT, g->d_adv_coef, g->d_mass, g->d_temp, g->d_mob, g->d_diff,
                 g->d_rate, g->d_HL, g->d_GL, g->d_CA, g->d_CB, g->d_tri};
    k_export<<<(unsigned)((need + 255) / 256), 256, 0, (cudaStream_t)stream>>>(v, which, out, need);
    CUDA_OR_FAIL(cudaGetLastError(), "k_export");
    return BTE_OK;
}

int bte_initialize(const bte_grid* g, int P, double* f, void* stream) {
    if (!g || !f || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P == 0) return BTE_OK;
    cudaSetDevice(g->device);
    cudaStream_t s = (cudaStream_t)stream;
    // angular factor: 2-point Gauss-Legendre in cos(theta) times the 2-point periodic
    // trapezoid in phi (function_to_basis with NUM_Q_VT = NUM_Q_VP = 2)
    std::vector<double> gx, gw;
    gauss_legendre(2, gx, gw);
    std::vector<double> ang(g->nsh, 0.0);
    for (int l = 0; l < g->nsh; ++l) {
        double acc = 0.0;
        for (int i = 0; i < 2; ++i) {
            double mu = std::cos(std::acos(gx[i]));
            double p0 = 1.0, p1 = mu, P = (l == 0) ? 1.0 : mu;
            for (int k = 2; k <= l; ++k) { P = ((2.0 * k - 1.0) * mu * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = P; }
            acc += std::sqrt((2.0 * l + 1) / (4.0 * M_PI)) * P * gw[i];
        }
        ang[l] = acc * (2.0 * M_PI / 2.0) * 2.0;
    }
    double *radial = nullptr, *dang = nullptr;
    CUDA_OR_FAIL(cudaMallocAsync((void**)&radial, g->nsp * sizeof(double), s), "alloc");
    CUDA_OR_FAIL(cudaMallocAsync((void**)&dang, g->nsh * sizeof(double), s), "alloc");
    CUDA_OR_FAIL(cudaMemcpyAsync(dang, ang.data(), g->nsh * sizeof(double), cudaMemcpyHostToDevice, s), "copy");
    k_maxwell_rhs<<<(g->nsp + 127) / 128, 128, 0, s>>>(g->nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span,
                                                      g->q5.B, radial);
    k_maxwell_fill<<<(g->n + 127) / 128, 128, 0, s>>>(g->nsp, g->nsh, g->d_Minv, radial, dang, f, P);
    CUDA_OR_FAIL(cudaGetLastError(), "k_maxwell");
    cudaFreeAsync(radial, s);
    cudaFreeAsync(dang, s);
    CUDA_OR_FAIL(cudaStreamSynchronize(s), "initialize");
    return BTE_OK;
}

} // extern "C"

// Scratch of bte_initialize_noalloc: the radial projection of the Maxwellian (n_sp doubles,
// from offset 0) and the angular factors (num_sh doubles, from offset
// BTE_INIT_NOALLOC_MAX_NSP). Static device memory of this module, so every GPU that loads
// the library holds these 4,160 bytes until the process exits. Host code must not pass
// `g_init_scratch` itself to a kernel (on the host it names a stand-in, not device memory):
// it passes the address that init_scratch_address looked up.
static __device__ __align__(256) double g_init_scratch[BTE_INIT_NOALLOC_MAX_NSP + BTE_INIT_NOALLOC_MAX_SH];
static_assert(BTE_INIT_NOALLOC_MAX_NSP == 512 && BTE_INIT_NOALLOC_MAX_SH == 8, "limits quoted in messages");
#define BTE_NOALLOC_MAX_DEVICES 64
static double* g_init_scratch_ptr[BTE_NOALLOC_MAX_DEVICES];
static std::mutex g_init_scratch_mu;

// Device address of g_init_scratch on `device` (which must be current); looked up once per
// device on its first use, and cached.
static int init_scratch_address(int device, double** out) {
    if (device < 0 || device >= BTE_NOALLOC_MAX_DEVICES)
        return fail(BTE_ERR_ARG, "bte_initialize_noalloc: device index beyond the library's table of 64 devices");
    std::lock_guard<std::mutex> lock(g_init_scratch_mu);
    if (!g_init_scratch_ptr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_init_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "bte_initialize_noalloc: cudaGetSymbolAddress of the scratch");
        g_init_scratch_ptr[device] = (double*)ptr;
    }
    *out = g_init_scratch_ptr[device];
    return BTE_OK;
}

extern "C" {

int bte_initialize_noalloc(const bte_grid* g, int P, double* f, void* stream) {
    if (!g || !f || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (g->nsp > BTE_INIT_NOALLOC_MAX_NSP || g->nsh > BTE_INIT_NOALLOC_MAX_SH)
        return fail(BTE_ERR_ARG, "bte_initialize_noalloc: grid too large for the static scratch "
                                 "(needs n_sp <= 512 and num_sh <= 8); use bte_initialize");
    if (P == 0) return BTE_OK;
    CUDA_OR_FAIL(cudaSetDevice(g->device), "cudaSetDevice");
    double* scratch = nullptr;
    int rc = init_scratch_address(g->device, &scratch);
    if (rc != BTE_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // angular factors on the host stack: the 2-point Gauss-Legendre rule in cos(theta)
    // (nodes -+1/sqrt(3), weights 1) times the 2-point periodic trapezoid in phi
    double ang[BTE_INIT_NOALLOC_MAX_SH];
    const double node = 1.0 / std::sqrt(3.0);
    for (int l = 0; l < g->nsh; ++l) {
        double acc = 0.0;
        for (int i = 0; i < 2; ++i) {
            const double mu = (i == 0) ? -node : node;
            double p0 = 1.0, p1 = mu, Pl = (l == 0) ? 1.0 : mu;
            for (int k = 2; k <= l; ++k) { Pl = ((2.0 * k - 1.0) * mu * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = Pl; }
            acc += std::sqrt((2.0 * l + 1) / (4.0 * M_PI)) * Pl;
        }
        ang[l] = acc * (2.0 * M_PI / 2.0) * 2.0;
    }
    // both scratch regions are written in full (radial by k_maxwell_rhs, ang by the copy)
    // before they are read, so nothing left by an earlier call needs clearing
    double* radial = scratch;
    double* dang = scratch + BTE_INIT_NOALLOC_MAX_NSP;
    CUDA_OR_FAIL(cudaMemcpyAsync(dang, ang, g->nsh * sizeof(double), cudaMemcpyHostToDevice, s), "copy");
    k_maxwell_rhs<<<(g->nsp + 127) / 128, 128, 0, s>>>(g->nsp, g->d_span_iv, g->q5.q, g->q5.x, g->q5.w, g->q5.span,
                                                      g->q5.B, radial);
    k_maxwell_fill<<<(g->n + 127) / 128, 128, 0, s>>>(g->nsp, g->nsh, g->d_Minv, radial, dang, f, P);
    CUDA_OR_FAIL(cudaGetLastError(), "k_maxwell");
    CUDA_OR_FAIL(cudaStreamSynchronize(s), "initialize");
    return BTE_OK;
}

int bte_engine_create(bte_grid* g, int capacity, int fp64_capacity, const bte_solve_opts* opts, bte_engine** out) {
    if (!g || !opts || !out) return fail(BTE_ERR_ARG, "null argument");
    *out = nullptr;
    if (capacity < 1 || capacity > (1 << 20)) return fail(BTE_ERR_ARG, "capacity out of range [1, 2^20]");
    if (opts->precision != BTE_PREC_FP64 && opts->precision != BTE_PREC_MIXED) return fail(BTE_ERR_ARG, "bad precision");
    if (opts->max_iter < 1 || !(opts->alpha_rho > 0 && opts->alpha_rho < 1)) return fail(BTE_ERR_ARG, "bad solver options");
    if (opts->precision == BTE_PREC_MIXED && fp64_capacity < 1) return fail(BTE_ERR_ARG, "the mixed form needs fp64_capacity >= 1");
    CUDA_OR_FAIL(cudaSetDevice(g->device), "cudaSetDevice");
    int rc = bte_engine_create_impl(g, capacity, fp64_capacity, opts, out);
    if (rc != BTE_OK) return fail(rc, rc == BTE_ERR_ALLOC ? "engine: device allocation failed" : "engine: create failed");
    return BTE_OK;
}

int bte_engine_destroy(bte_engine* e) {
    if (!e) return BTE_OK;
    cudaSetDevice(bte_engine_grid(e)->device);
    cudaDeviceSynchronize();
    bte_engine_destroy_impl(e);
    return BTE_OK;
}

int bte_engine_admit(bte_engine* e, int P, const double* n0, const double* ne, const double* ns_by_n0,
                     const double* Tg, const double* E, const double* f0, int ee, int32_t* slots, void* stream) {
    if (!e || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P == 0) return BTE_OK;
    if (!n0 || !ne || !ns_by_n0 || !Tg || !E || !f0 || !slots) return fail(BTE_ERR_ARG, "null buffer");
    BteGrid* g = bte_engine_grid(e);
    if (ee && !g->ee) return fail(BTE_ERR_STATE, "e-e requested but the grid was built without Coulomb operators");
    if (P > bte_engine_free_slots(e)) return fail(BTE_ERR_STATE, "not enough free slots");
    cudaSetDevice(g->device);
    int rc = bte_engine_admit_impl(e, P, n0, ne, ns_by_n0, Tg, E, f0, ee, slots, (cudaStream_t)stream);
    if (rc != BTE_OK) return fail(rc, std::string("engine admit failed: ") + cudaGetErrorString(cudaGetLastError()));
    return BTE_OK;
}

int bte_engine_step(bte_engine* e, int* n_done, int32_t* done_slots, void* stream) {
    if (!e || !n_done || !done_slots) return fail(BTE_ERR_ARG, "null argument");
    cudaSetDevice(bte_engine_grid(e)->device);
    int rc = bte_engine_step_impl(e, n_done, done_slots, (cudaStream_t)stream);
    if (rc != BTE_OK) return fail(rc, std::string("engine step failed: ") + cudaGetErrorString(cudaGetLastError()));
    return BTE_OK;
}

int bte_engine_collect(bte_engine* e, int P, const int32_t* slots, double* f, int32_t* status, int32_t* iters,
                       void* stream) {
    if (!e || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P == 0) return BTE_OK;
    if (!slots || !f) return fail(BTE_ERR_ARG, "null buffer");
    cudaSetDevice(bte_engine_grid(e)->device);
    int rc = bte_engine_collect_impl(e, P, slots, f, status, iters, (cudaStream_t)stream);
    if (rc == BTE_ERR_ARG) return fail(rc, "slot index out of range");
    if (rc != BTE_OK) return fail(rc, std::string("engine collect failed: ") + cudaGetErrorString(cudaGetLastError()));
    return BTE_OK;
}

int bte_engine_info(const bte_engine* e, int* ints4, size_t* bytes) {
    if (!e || !ints4) return fail(BTE_ERR_ARG, "null argument");
    ints4[0] = bte_engine_capacity(e);
    ints4[1] = bte_engine_free_slots(e);
    ints4[2] = bte_engine_active(e);
    ints4[3] = bte_engine_fp64_capacity(e);
    if (bytes) *bytes = bte_engine_bytes(e);
    return BTE_OK;
}

int bte_solve_transient(bte_grid* g, int P, const double* n0, const double* ne, const double* ns_by_n0,
                        const double* Tg, const double* E, const double* eRe, const double* eIm, double* f,
                        double* f_avg, int32_t* status, int32_t* iters, const bte_transient_opts* opts, void* stream) {
    if (!g || !opts || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P == 0) return BTE_OK;
    if (!n0 || !ne || !ns_by_n0 || !Tg || !E || !f || !status || !iters) return fail(BTE_ERR_ARG, "null buffer");
    if (opts->efreq > 0 && (!eRe || !eIm)) return fail(BTE_ERR_ARG, "eRe and eIm are needed with a field frequency");
    if (opts->precision != BTE_PREC_FP64 && opts->precision != BTE_PREC_MIXED) return fail(BTE_ERR_ARG, "bad precision");
    if (!(opts->dt > 0) || !(opts->cycles >= 0) || opts->max_iter < 1 || opts->efreq < 0)
        return fail(BTE_ERR_ARG, "bad transient options");
    if (opts->ee && !g->ee) return fail(BTE_ERR_STATE, "e-e requested but the grid was built without Coulomb operators");
    cudaSetDevice(g->device);
    int rc = bte_transient_impl(g, P, n0, ne, ns_by_n0, Tg, E, eRe, eIm, f, f_avg, status, iters, opts,
                                (cudaStream_t)stream);
    if (rc == BTE_ERR_STATE) return fail(rc, "a transient step did not converge within max_iter chord iterations");
    if (rc != BTE_OK) return fail(rc, std::string("transient solve failed: ") + cudaGetErrorString(cudaGetLastError()));
    return BTE_OK;
}

int bte_solve_steady(bte_grid* g, int P, const double* n0, const double* ne, const double* ns_by_n0, const double* Tg,
                     const double* E, double* f, int32_t* status, int32_t* iters, const bte_solve_opts* opts,
                     void* stream) {
    if (!g || !opts || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P > 0 && (!n0 || !ne || !ns_by_n0 || !Tg || !E || !f || !status || !iters)) return fail(BTE_ERR_ARG, "null buffer");
    if (opts->precision != BTE_PREC_FP64 && opts->precision != BTE_PREC_MIXED) return fail(BTE_ERR_ARG, "bad precision");
    if (opts->max_iter < 0 || !(opts->alpha_rho > 0 && opts->alpha_rho < 1)) return fail(BTE_ERR_ARG, "bad solver options");
    if (opts->ee && !g->ee) return fail(BTE_ERR_STATE, "e-e requested but the grid was built without Coulomb operators");
    cudaSetDevice(g->device);
    int rc = bte_solve_impl(g, P, n0, ne, ns_by_n0, Tg, E, f, status, iters, opts, (cudaStream_t)stream);
    if (rc != BTE_OK) {
        cudaError_t e = cudaGetLastError();
        return fail(rc, std::string("solve failed: ") + cudaGetErrorString(e));
    }
    CUDA_OR_FAIL(cudaStreamSynchronize((cudaStream_t)stream), "solve");
    return BTE_OK;
}

int bte_solve_info(bte_grid* g, int P, double* r_final, double* r_initial, void* stream) {
    if (!g || P < 0 || !r_final || !r_initial) return fail(BTE_ERR_ARG, "bad argument");
    cudaSetDevice(g->device);
    int rc = bte_solve_info_impl(g, P, r_final, r_initial, (cudaStream_t)stream);
    if (rc) return fail(rc, "no steady solve of that size has run on this grid");
    return BTE_OK;
}

int bte_qoi(const bte_grid* g, int P, const double* f, const double* n0, const double* E, int effective_mobility,
            double* energy, double* mobility, double* diffusion, double* rates, void* stream) {
    if (!g || P < 0) return fail(BTE_ERR_ARG, "bad argument");
    if (P == 0) return BTE_OK;
    if (!f || !n0 || !E || !energy || !mobility || !diffusion || !rates) return fail(BTE_ERR_ARG, "null buffer");
    cudaSetDevice(g->device);
    k_qoi<<<(P + 127) / 128, 128, 0, (cudaStream_t)stream>>>(g->nsp, g->nsh, g->nproc, g->mw0, g->vth, g->d_mass,
                                                             g->d_temp, g->d_mob, g->d_diff, g->d_rate, f, n0, E,
                                                             effective_mobility, energy, mobility, diffusion, rates, P);
    CUDA_OR_FAIL(cudaGetLastError(), "k_qoi");
    return BTE_OK;
}

int bte_lu_factor(int dtype, int P, int N, void* A, int ld, long long stride, int32_t* piv, int32_t* info,
                  void* stream) {
    return bte_lu_factor_ex(dtype, P, N, A, ld, stride, piv, info, 0, stream);
}

int bte_lu_factor_ex(int dtype, int P, int N, void* A, int ld, long long stride, int32_t* piv, int32_t* info,
                     int kernel, void* stream) {
    if (P < 0 || N < 1 || N > 2048 || ld < N || stride < (long long)ld * N || !A || !piv || !info || kernel < 0 ||
        kernel > 6)
        return fail(BTE_ERR_ARG, "bad LU arguments");
    if ((kernel == 2 || kernel == 4 || kernel == 5) && (dtype == 0 || N > 512))
        return fail(BTE_ERR_ARG, "the tensor-core LU is FP32 with N <= 512");
    if (kernel == 3 && N > 512) return fail(BTE_ERR_ARG, "the left-looking LU takes N <= 512");
    if (kernel == 6 && dtype != 0) return fail(BTE_ERR_ARG, "the split LU is FP64");
    cudaError_t e = (dtype == 0)
                        ? bte_lu_factor_t<double>(P, N, N, (double*)A, ld, stride, piv, info, (cudaStream_t)stream, kernel)
                        : bte_lu_factor_t<float>(P, N, N, (float*)A, ld, stride, piv, info, (cudaStream_t)stream, kernel);
    CUDA_OR_FAIL(e, "bte_lu_factor");
    return BTE_OK;
}

int bte_lu_solve(int dtype, int P, int N, const void* A, int ld, long long stride, const int32_t* piv, void* b,
                 void* stream) {
    if (P < 0 || N < 1 || ld < N || !A || !piv || !b) return fail(BTE_ERR_ARG, "bad LU arguments");
    cudaError_t e = (dtype == 0)
                        ? bte_lu_solve_t<double>(P, N, (const double*)A, ld, stride, piv, (double*)b, 0, (cudaStream_t)stream)
                        : bte_lu_solve_t<float>(P, N, (const float*)A, ld, stride, piv, (float*)b, 0, (cudaStream_t)stream);
    CUDA_OR_FAIL(e, "bte_lu_solve");
    return BTE_OK;
}

}  // extern "C"
