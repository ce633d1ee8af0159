// Host build of the finite-volume 1D3V fully implicit step's shared core
// (boltzmann_gb300/csrc/fvm_core.h): the same per-element operator and collision-inverse
// arithmetic and the same GMRES loop the CUDA kernels run, driven by host loops, so that the
// tests compare them with the oracle without a GPU. The op-split sweeps are plain host line
// solves here (the library's sweep kernels are checked on the GPU against the oracle).
// Built by tests/test_fvm_core_host.py with the host C++ compiler into a temporary directory.
#include <string.h>

#include <vector>

#include "fvm_core.h"

namespace {

struct Setup {
    FvmView v;
    std::vector<int8_t> north;
    std::vector<double> cth;
    const double* gain;
    const double* vt;
};

Setup make_setup(int Nr, int Nvt, int Nx, int ndr, int ndt, int ndx, const double* vr, const double* vt,
                 const double* w, const double* loss, const double* gain, const double* const* bands) {
    Setup s;
    s.north.resize(Nvt);
    s.cth.resize(Nvt);
    for (int j = 0; j < Nvt; ++j) {
        s.cth[j] = cos(vt[j]);
        s.north[j] = vt[j] <= 0.5 * 3.14159265358979323846 ? 1 : 0;
    }
    s.v.Nr = Nr; s.v.Nvt = Nvt; s.v.Nx = Nx; s.v.ndr = ndr; s.v.ndt = ndt; s.v.ndx = ndx;
    s.v.vr = vr; s.v.cos_t = s.cth.data(); s.v.north = s.north.data(); s.v.w = w; s.v.loss = loss;
    s.v.vrL = bands[0]; s.v.vrR = bands[1]; s.v.vtL = bands[2]; s.v.vtR = bands[3]; s.v.xL = bands[4]; s.v.xR = bands[5];
    s.gain = gain;
    s.vt = vt;
    return s;
}

// T = A m, A (Nr x Nr), m (Nr x Nx) the ordinate moments of X
void moments_times(const FvmView& v, const double* A, const double* X, std::vector<double>& T) {
    std::vector<double> m((size_t)v.Nr * v.Nx);
    for (int r = 0; r < v.Nr; ++r)
        for (int x = 0; x < v.Nx; ++x) m[(size_t)r * v.Nx + x] = fvm_moment_at(v, X, r, x);
    T.assign((size_t)v.Nr * v.Nx, 0.0);
    for (int r = 0; r < v.Nr; ++r)
        for (int q = 0; q < v.Nr; ++q)
            for (int x = 0; x < v.Nx; ++x) T[(size_t)r * v.Nx + x] += A[(size_t)r * v.Nr + q] * m[(size_t)q * v.Nx + x];
}

void mvec(const Setup& s, const FvmCoef& c, const double* E, const double* X, double* Y) {
    const FvmView& v = s.v;
    std::vector<double> G;
    moments_times(v, s.gain, X, G);
    for (int r = 0; r < v.Nr; ++r)
        for (int j = 0; j < v.Nvt; ++j)
            for (int x = 0; x < v.Nx; ++x)
                Y[((size_t)r * v.Nvt + j) * v.Nx + x] = fvm_mvec_at(v, c, E, G.data(), X, r, j, x);
}

// (I + a h D) o = b along a line of N values at stride st; D the column-stored lower band L
// (left to right) when ltr, else the upper band R
void line_solve(const double* L, const double* R, int nd, int N, double a, bool ltr, double h, double* y, long long st) {
    const double ad = a * h;
    std::vector<double> o(N), b(N);
    for (int i = 0; i < N; ++i) b[i] = y[(long long)i * st];
    if (ltr) {
        for (int i = 0; i < N; ++i) {
            double acc = 0.0;
            for (int k = 1; k < nd && k <= i; ++k) acc += L[(size_t)k * N + (i - k)] * o[i - k];
            o[i] = (b[i] - ad * acc) / (1.0 + ad * L[i]);
        }
    } else {
        for (int i = N - 1; i >= 0; --i) {
            double acc = 0.0;
            for (int k = 1; k < nd && i + k < N; ++k) acc += R[(size_t)k * N + (i + k)] * o[i + k];
            o[i] = (b[i] - ad * acc) / (1.0 + ad * R[i]);
        }
    }
    for (int i = 0; i < N; ++i) y[(long long)i * st] = o[i];
}

void precond(const Setup& s, const double* dinv, const double* H, double cE, double ax, double h, const double* E,
             const double* X, double* Y) {
    const FvmView& v = s.v;
    const int Nr = v.Nr, Nvt = v.Nvt, Nx = v.Nx;
    std::vector<double> T;
    moments_times(v, H, X, T);
    for (int r = 0; r < Nr; ++r)
        for (int j = 0; j < Nvt; ++j)
            for (int x = 0; x < Nx; ++x)
                Y[((size_t)r * Nvt + j) * Nx + x] = fvm_coll_apply_at(v, dinv, T.data(), X, r, j, x);
    for (int x = 0; x < Nx; ++x)   // v_r lines, a = -aE cos(theta_j), left to right when a >= 0
        for (int j = 0; j < Nvt; ++j) {
            const double a = -(cE * E[x]) * v.cos_t[j];
            line_solve(v.vrL, v.vrR, v.ndr, Nr, a, a >= 0.0, h, Y + (size_t)j * Nx + x, (long long)Nvt * Nx);
        }
    for (int x = 0; x < Nx; ++x)   // v_theta lines, a = aE / v_r, left to right when -a >= 0
        for (int r = 0; r < Nr; ++r) {
            const double a = (cE * E[x]) / v.vr[r];
            line_solve(v.vtL, v.vtR, v.ndt, Nvt, a, -a >= 0.0, h, Y + (size_t)r * Nvt * Nx + x, Nx);
        }
    for (int r = 0; r < Nr; ++r)
        for (int j = 0; j < Nvt; ++j) {
            double* line = Y + ((size_t)r * Nvt + j) * Nx;
            line[v.north[j] ? 0 : Nx - 1] = 0.0;
            const double a = (ax * v.vr[r]) * v.cos_t[j];
            line_solve(v.xL, v.xR, v.ndx, Nx, a, a >= 0.0, h, line, 1);
        }
}

struct HostOps {
    const Setup* s;
    FvmCoef c;
    const double* E;
    const double *dinv, *H;
    double cE, hstep;
    size_t N;
    double *B, *X, *R, *W, *Z, *T, *Kr;
    bool identity;
    int matvec(const double* x, double* y) { mvec(*s, c, E, x, y); return 0; }
    int precond(const double* x, double* y) {
        if (identity) { memcpy(y, x, N * sizeof(double)); return 0; }
        std::vector<double> tmp(x, x + N);
        ::precond(*s, dinv, H, cE, c.ax, hstep, E, tmp.data(), y);
        return 0;
    }
    int dots(int k, const double* V, const double* w, double* out) {
        for (int j = 0; j < k; ++j) {
            double acc = 0.0;
            for (size_t i = 0; i < N; ++i) acc += V[(size_t)j * N + i] * w[i];
            out[j] = acc;
        }
        return 0;
    }
    int sub_combo(int k, const double* V, const double* h, double* w) {
        for (size_t i = 0; i < N; ++i) {
            double acc = w[i];
            for (int j = 0; j < k; ++j) acc -= h[j] * V[(size_t)j * N + i];
            w[i] = acc;
        }
        return 0;
    }
    int combo(int k, const double* V, const double* cc, double* y) {
        for (size_t i = 0; i < N; ++i) {
            double acc = 0.0;
            for (int j = 0; j < k; ++j) acc += cc[j] * V[(size_t)j * N + i];
            y[i] = acc;
        }
        return 0;
    }
    int scale(double a, const double* x, double* y) { for (size_t i = 0; i < N; ++i) y[i] = a * x[i]; return 0; }
    int axpy(double a, const double* x, double* y) { for (size_t i = 0; i < N; ++i) y[i] += a * x[i]; return 0; }
    int sub(const double* a, const double* b, double* cc) { for (size_t i = 0; i < N; ++i) cc[i] = a[i] - b[i]; return 0; }
};

// a dense operator with a diagonal preconditioner, for the solver alone
struct DenseOps {
    size_t N;
    const double* A;      // N x N row-major
    const double* minv;   // N: the preconditioner's diagonal
    double *B, *X, *R, *W, *Z, *T, *Kr;
    int matvec(const double* x, double* y) {
        for (size_t i = 0; i < N; ++i) {
            double acc = 0.0;
            for (size_t j = 0; j < N; ++j) acc += A[i * N + j] * x[j];
            y[i] = acc;
        }
        return 0;
    }
    int precond(const double* x, double* y) { for (size_t i = 0; i < N; ++i) y[i] = minv[i] * x[i]; return 0; }
    int dots(int k, const double* V, const double* w, double* out) {
        for (int j = 0; j < k; ++j) {
            double acc = 0.0;
            for (size_t i = 0; i < N; ++i) acc += V[(size_t)j * N + i] * w[i];
            out[j] = acc;
        }
        return 0;
    }
    int sub_combo(int k, const double* V, const double* h, double* w) {
        for (size_t i = 0; i < N; ++i)
            for (int j = 0; j < k; ++j) w[i] -= h[j] * V[(size_t)j * N + i];
        return 0;
    }
    int combo(int k, const double* V, const double* cc, double* y) {
        for (size_t i = 0; i < N; ++i) {
            double acc = 0.0;
            for (int j = 0; j < k; ++j) acc += cc[j] * V[(size_t)j * N + i];
            y[i] = acc;
        }
        return 0;
    }
    int scale(double a, const double* x, double* y) { for (size_t i = 0; i < N; ++i) y[i] = a * x[i]; return 0; }
    int axpy(double a, const double* x, double* y) { for (size_t i = 0; i < N; ++i) y[i] += a * x[i]; return 0; }
    int sub(const double* a, const double* b, double* cc) { for (size_t i = 0; i < N; ++i) cc[i] = a[i] - b[i]; return 0; }
};

FvmCoef coef(const double* c6) {
    FvmCoef c;
    c.dt = c6[0]; c.dtx = c6[1]; c.tau = c6[2]; c.kappa = c6[3]; c.cA = c6[4]; c.ax = c6[5];
    return c;
}

}  // namespace

extern "C" {

// dims: Nr, Nvt, Nx, ndr, ndt, ndx; bands: the six column-stored bands; c6: dt, dtx, tau, kappa, cA, ax
void fvm_host_mvec(const int* dims, const double* vr, const double* vt, const double* w, const double* loss,
                   const double* gain, const double* const* bands, const double* c6, const double* E, const double* X,
                   double* Y) {
    Setup s = make_setup(dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], vr, vt, w, loss, gain, bands);
    mvec(s, coef(c6), E, X, Y);
}

void fvm_host_precond(const int* dims, const double* vr, const double* vt, const double* w, const double* loss,
                      const double* gain, const double* const* bands, const double* dinv, const double* H, double cE,
                      double ax, double hstep, const double* E, const double* X, double* Y) {
    Setup s = make_setup(dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], vr, vt, w, loss, gain, bands);
    precond(s, dinv, H, cE, ax, hstep, E, X, Y);
}

// the solver alone on a dense system A x = b with the preconditioner diag(minv); x out
int gmres_host_dense(int n, const double* A, const double* minv, const double* b, double* x, int restart, double rtol,
                     double atol, int max_iter, int pc_left, double* info4) {
    const size_t N = (size_t)n;
    std::vector<double> B(b, b + N), X(N), R(N), W(N), Z(N), T(N), Kr((size_t)(restart + 1) * N);
    DenseOps op{N, A, minv, B.data(), X.data(), R.data(), W.data(), Z.data(), T.data(), Kr.data()};
    FvmGmresInfo info{};
    const int rc = pc_left ? fvm_gmres_left(op, restart, rtol, atol, max_iter, &info)
                           : fvm_gmres(op, restart, rtol, atol, max_iter, &info);
    memcpy(x, X.data(), N * sizeof(double));
    info4[0] = info.iterations;
    info4[1] = info.rnorm;
    info4[2] = info.bnorm > 0.0 ? info.rnorm / info.bnorm : 0.0;
    info4[3] = info.converged ? 0.0 : 1.0;
    return rc;
}

// the semi-Lagrangian advection: Y = step_adv_vx_sl(V); dims: Nr, Nvt, Nx
void fvm_host_sl(const int* dims, const double* vr, const double* vt, const double* x, double vmin, double vmax,
                 double cX, double cE, const double* E, const double* V, double* Y) {
    const int Nr = dims[0], Nvt = dims[1], Nx = dims[2];
    std::vector<double> cth(Nvt), vrp(Nr + 2), vta(Nvt + 2);
    for (int j = 0; j < Nvt; ++j) cth[j] = cos(vt[j]);
    vrp[0] = vmin;
    vrp[Nr + 1] = vmax;
    for (int r = 0; r < Nr; ++r) vrp[r + 1] = vr[r];
    vta[0] = 0.0;
    vta[Nvt + 1] = 3.14159265358979323846;
    for (int j = 0; j < Nvt; ++j) vta[j + 1] = vt[Nvt - 1 - j];
    FvmSl s;
    s.Nr = Nr; s.Nvt = Nvt; s.Nx = Nx; s.vr = vr; s.vt = vt; s.cos_t = cth.data(); s.vrp = vrp.data();
    s.vta = vta.data(); s.x = x; s.vmin = vmin; s.cX = cX; s.cE = cE;
    for (int r = 0; r < Nr; ++r)
        for (int j = 0; j < Nvt; ++j)
            for (int i = 0; i < Nx; ++i) Y[((size_t)r * Nvt + j) * Nx + i] = fvm_sl_at(s, E, V, r, j, i);
}

// V replaced by the step's solution; info4 as bte_fvm_step's
int fvm_host_step(const int* dims, const double* vr, const double* vt, const double* w, const double* loss,
                  const double* gain, const double* const* bands, const double* dinv, const double* H, const double* c6,
                  double alpha, int pc_mode, const double* E, double* V, double rtol, double atol, int restart,
                  int max_iter, double* info4) {
    Setup s = make_setup(dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], vr, vt, w, loss, gain, bands);
    const FvmCoef c = coef(c6);
    const size_t N = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<double> B(V, V + N), X(N), R(N), W(N), Z(N), T(N), Kr((size_t)(restart + 1) * N);
    for (int r = 0; r < dims[0]; ++r)
        for (int j = 0; j < dims[1]; ++j) B[((size_t)r * dims[1] + j) * dims[2] + (s.north[j] ? 0 : dims[2] - 1)] = 0.0;
    HostOps op{&s, c, E, dinv, H, c.tau * c.cA, alpha * c.dt, N, B.data(), X.data(), R.data(), W.data(), Z.data(),
               T.data(), Kr.data(), pc_mode == 2};
    FvmGmresInfo info{};
    const int rc = pc_mode == 1 ? fvm_gmres_left(op, restart, rtol, atol, max_iter, &info)
                                : fvm_gmres(op, restart, rtol, atol, max_iter, &info);
    memcpy(V, X.data(), N * sizeof(double));
    info4[0] = info.iterations;
    info4[1] = info.rnorm;
    info4[2] = info.bnorm > 0.0 ? info.rnorm / info.bnorm : 0.0;
    info4[3] = info.converged ? 0.0 : 1.0;
    return rc;
}

}  // extern "C"
