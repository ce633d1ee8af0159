// Double-double accumulation of products: (hi, lo) += a * b with the product split exactly by
// an fma (TwoProduct) and the sum by Knuth's TwoSum, the low parts gathered in lo and the pair
// left unnormalised (hi + lo is the value). Used by the residual of a point at its FP64
// rounding floor (newton.cu, residual_row_dd); compiled for the host by the CPU tests
// (tests/host/dd_harness.cpp), hence no CUDA-only constructs.
#pragma once
#include <cmath>

#if defined(__CUDACC__)
#define BTE_DD_HD __host__ __device__
#else
#define BTE_DD_HD
#endif

BTE_DD_HD inline void dd_acc(double& hi, double& lo, double a, double b) {
    const double pr = a * b;
#if defined(__CUDA_ARCH__)
    const double pe = fma(a, b, -pr);
#else
    const double pe = std::fma(a, b, -pr);
#endif
    const double sm = hi + pr, v = sm - hi, e = (hi - (sm - v)) + (pr - v);
    hi = sm;
    lo += e + pe;
}

// (hi, lo) += (ahi + alo) * b
BTE_DD_HD inline void dd_acc2(double& hi, double& lo, double ahi, double alo, double b) {
    dd_acc(hi, lo, ahi, b);
    lo += alo * b;
}
