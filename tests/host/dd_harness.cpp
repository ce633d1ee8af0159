// Host build of the library's double-double accumulation (boltzmann_gb300/csrc/dd_arith.h)
// for the CPU tests: dd_dot(n, a, b, out) writes hi and lo of sum_i a[i] * b[i].
#include "../../boltzmann_gb300/csrc/dd_arith.h"

extern "C" void dd_dot(int n, const double* a, const double* b, double* out) {
    double hi = 0.0, lo = 0.0;
    for (int i = 0; i < n; ++i) dd_acc(hi, lo, a[i], b[i]);
    out[0] = hi;
    out[1] = lo;
}

// (hi, lo) of sum_i (ahi[i] + alo[i]) * b[i]
extern "C" void dd_dot2(int n, const double* ahi, const double* alo, const double* b, double* out) {
    double hi = 0.0, lo = 0.0;
    for (int i = 0; i < n; ++i) dd_acc2(hi, lo, ahi[i], alo[i], b[i]);
    out[0] = hi;
    out[1] = lo;
}
