// Host build of afmibins_gb300/csrc/dfloat.cuh for the CPU tests: the
// block-floating-point residuals and the double-float helpers, exported with
// C linkage so that the tests can compare them with exact rational arithmetic.
#define __host__
#define __device__
#define __forceinline__ inline
#include <cmath>
#include <cstring>
using std::fmaf;
#include "dfloat.cuh"

extern "C" {
float afmib_test_helm_residual(double b, double x0, const double* nb, const int* cnb, int nnb, int coef0, double f) {
    return afmib::helm_residual_bfp(b, x0, nb, cnb, nnb, coef0, afmib::df_split(f));
}
float afmib_test_lap_residual(double b, double x0, const double* nb, int nnb, int c, int k2) {
    return afmib::lap_residual_bfp(b, x0, nb, nnb, c, k2);
}
float afmib_test_df_round(double d) { return afmib::df_round(d); }
void afmib_test_split_round(double d, float* hi, float* lo) {
    const afmib::df2 r = afmib::df_split_round(d);
    *hi = r.hi;
    *lo = r.lo;
}
// sin(pi x), cos(pi x) of df_sincospi for x (split by df_split), as pairs
void afmib_test_sincospi(double x, float* s, float* c) {
    afmib::df2 sp, cp;
    afmib::df_sincospi(afmib::df_split(x), &sp, &cp);
    s[0] = sp.hi;
    s[1] = sp.lo;
    c[0] = cp.hi;
    c[1] = cp.lo;
}
void afmib_test_split(double d, float* hi, float* lo) {
    const afmib::df2 r = afmib::df_split(d);
    *hi = r.hi;
    *lo = r.lo;
}
// count of inputs (out of n, from a small LCG over raw bit patterns plus the
// edge cases) where the integer FP32 -> FP64 conversion differs from the C cast
long long afmib_test_convert_mismatches(long long n, unsigned long long seed) {
    long long bad = 0;
    unsigned long long st = seed;
    auto next = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return st;
    };
    auto same32 = [](float a, float b) { return std::memcmp(&a, &b, 4) == 0 || (a != a && b != b); };
    auto same64 = [](double a, double b) { return std::memcmp(&a, &b, 8) == 0 || (a != a && b != b); };
    auto check = [&](double v) {
        const float f = (float)v;
        if (!same64(afmib::f32_to_f64(f), (double)f)) ++bad;
        float g;
        const unsigned w = (unsigned)(v == v ? afmib::dbits(v) >> 16 : 0x7fc00001u);  // raw float bit patterns too
        std::memcpy(&g, &w, 4);
        if (!same64(afmib::f32_to_f64(g), (double)g)) ++bad;
    };
    (void)same32;
    const double edges[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 3.40282357e38,
                            1.1754943508222875e-38, 1.1754942807573643e-38, 1.1754943e-38 * 0.5, 1e-300, -1e300,
                            1.0 + 1.0 / (1 << 24), 1.0 + 3.0 / (1 << 24), 1.0 - 1.0 / (1 << 25), 0.1, -2.5e-10};
    for (double v : edges) check(v);
    for (long long i = 0; i < n; ++i) {
        const unsigned long long r = next();
        switch (i % 4) {
            case 0: check(afmib::dfrom(r)); break;                              // any bit pattern
            case 1: check(afmib::dfrom((r & ~(0x7ffull << 52)) | ((896ull + (r >> 56) % 260) << 52))); break;  // float range
            case 2: check(afmib::dfrom((r & ~0x1FFFFFFFull) | 0x10000000ull)); break;  // exact ties
            default: check(afmib::dfrom(r | 0x1FFFFFFFull)); break;            // carries
        }
    }
    return bad;
}
void afmib_test_fixed(long long q, int E, float* hi, float* lo) {
    const afmib::df2 r = afmib::from_fixed(q, E);
    *hi = r.hi;
    *lo = r.lo;
}
}

extern "C" {
// r - H e for an FP32 correction e in double-float (df_helm_row), the FP64
// residual r given as its double-float pair (rh, rl); returns the new pair
void afmib_test_helm_update_df(float rh, float rl, float e0, const float* nb, int nnb, float k, double off, float xa,
                               double cxa, int wall, float* oh, float* ol) {
    afmib::df2 r;
    r.hi = rh;
    r.lo = rl;
    const afmib::df2 he = afmib::df_helm_row(e0, nb, nnb, k, afmib::df_split(off), xa, afmib::df_split(cxa), wall != 0);
    r = afmib::df_add(r, afmib::df_neg(he));
    *oh = r.hi;
    *ol = r.lo;
}
}

extern "C" {
// r - L e for an FP32 correction e in double-float (df_lap_row)
void afmib_test_lap_update_df(float rh, float rl, float e0, const float* nb, int nnb, float c, float off, float* oh,
                              float* ol) {
    afmib::df2 r;
    r.hi = rh;
    r.lo = rl;
    r = afmib::df_add(r, afmib::df_neg(afmib::df_lap_row(e0, nb, nnb, c, off)));
    *oh = r.hi;
    *ol = r.lo;
}
}

extern "C" {
float afmib_test_df_hi(double d) { return afmib::df_hi(d); }
}
