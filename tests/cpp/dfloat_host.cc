// Host build of afmibins_gb300/csrc/dfloat.cuh for the CPU tests: the
// block-floating-point residuals and the double-float helpers, exported with
// C linkage so that the tests can compare them with exact rational arithmetic.
#define __host__
#define __device__
#define __forceinline__ inline
#include <cmath>
using std::fmaf;
#include "dfloat.cuh"

extern "C" {
float afmib_test_helm_residual(double b, double x0, const double* nb, const int* cnb, int nnb, int coef0, double f) {
    return afmib::helm_residual_bfp(b, x0, nb, cnb, nnb, coef0, afmib::df_split(f));
}
float afmib_test_lap_residual(double b, double x0, const double* nb, int nnb, int c, int k2) {
    return afmib::lap_residual_bfp(b, x0, nb, nnb, c, k2);
}
void afmib_test_split(double d, float* hi, float* lo) {
    const afmib::df2 r = afmib::df_split(d);
    *hi = r.hi;
    *lo = r.lo;
}
void afmib_test_fixed(long long q, int E, float* hi, float* lo) {
    const afmib::df2 r = afmib::from_fixed(q, E);
    *hi = r.hi;
    *lo = r.lo;
}
}
