// Host-only harness: evaluates the library's B-spline and cross-section interpolation
// routines (bte_common.cuh) on the CPU so tests can compare them with SciPy.
// stdin: nsp, knots (nsp + 4), npts, points; then m, table x, table y, nq, queries.
// stdout: per point "span d0[4] d1[4] d2[4]", then the interpolated values.
#include <cstdio>
#include <vector>
#include "../../boltzmann_gb300/csrc/bte_common.cuh"

int main() {
    int nsp;
    if (scanf("%d", &nsp) != 1) return 1;
    std::vector<double> t(nsp + 4);
    for (auto& v : t) if (scanf("%lf", &v) != 1) return 1;
    int np_;
    if (scanf("%d", &np_) != 1) return 1;
    for (int i = 0; i < np_; ++i) {
        double x;
        if (scanf("%lf", &x) != 1) return 1;
        double d[3][4];
        int s = bspline_eval(t.data(), nsp, x, 2, d);
        printf("%d", s);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 4; ++b) printf(" %.17e", d[a][b]);
        printf("\n");
    }
    int m;
    if (scanf("%d", &m) != 1) return 1;
    std::vector<double> xs(m), ys(m);
    for (auto& v : xs) if (scanf("%lf", &v) != 1) return 1;
    for (auto& v : ys) if (scanf("%lf", &v) != 1) return 1;
    int nq;
    if (scanf("%d", &nq) != 1) return 1;
    for (int i = 0; i < nq; ++i) {
        double x;
        if (scanf("%lf", &x) != 1) return 1;
        printf("%.17e\n", interp_clamped(xs.data(), ys.data(), m, x));
    }
    return 0;
}
