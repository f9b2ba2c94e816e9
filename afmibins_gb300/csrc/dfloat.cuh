// Double-float ("df") arithmetic on the FP32 pipe for the FP64 outer
// residuals of the mixed form. On GB300 the FP64 pipe runs at 1/69 of the
// FP32 rate and every FP64<->FP32 conversion runs on it too, so an FP64
// 7-point residual is FP64-pipe bound at several times its HBM time. Here an
// FP64 word is split into two floats with integer operations only, and the
// stencil is evaluated with error-free transformations (Knuth's two-sum,
// the fused-multiply-add two-product) on pairs of floats.
//
// Precision: df_split keeps 24 + 23 significant bits (relative 2^-46, about
// 1.4e-14); df_add and df_mul are the accurate pair algorithms of
// Hida, Li and Bailey's double-double library restated for float pairs
// (relative error a few units of 2^-46). The residuals they produce carry
// rounding four or more orders below the solver tolerances (1e-10).
#pragma once

namespace afmib {

struct df2 {
    float hi, lo;
};

// hi = the top 24 significant bits of d (truncated), lo = the next 23, both
// with d's sign; |d| < 2^-126 (float subnormal range and zero) gives 0, and
// lo is dropped below 2^-80. No FP64 instruction is issued.
__device__ __forceinline__ df2 df_split(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned hw = (unsigned)(u >> 32), lw = (unsigned)u;
    const unsigned sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7ffu) - 1023;
    const unsigned mh = ((hw & 0xfffffu) << 3) | (lw >> 29);  // mantissa bits 51..29
    const unsigned ml = (lw >> 6) & 0x7fffffu;                 // mantissa bits 28..6
    df2 r;
    if (e < -126) {
        r.hi = 0.f;
        r.lo = 0.f;
        return r;
    }
    if (e > 127) {  // beyond the float range (and inf / nan): keep inf or nan
        r.hi = __int_as_float(sign | 0x7f800000u | (mh ? 0x400000u : 0u));
        r.lo = 0.f;
        return r;
    }
    r.hi = __int_as_float(sign | ((unsigned)(e + 127) << 23) | mh);
    const int el = e - 46;  // lo = ml * 2^(e - 46)
    if (el < -126 || ml == 0u) {
        r.lo = 0.f;
        return r;
    }
    const float m = __int_as_float(0x4B000000u | ml) - 8388608.0f;  // ml as a float, exactly
    const float sc = __int_as_float((unsigned)(el + 127) << 23);     // 2^el
    r.lo = __int_as_float(__float_as_int(m * sc) | sign);
    return r;
}

// a + b with both pairs' rounding errors carried (accurate under cancellation)
__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
    float s = a.hi + b.hi;
    float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);
    const float t = a.lo + b.lo;
    const float w = t - a.lo;
    const float f = (a.lo - (t - w)) + (b.lo - w);
    e += t;
    float h = s + e;
    e = e - (h - s);
    e += f;
    df2 r;
    r.hi = h + e;
    r.lo = e - (r.hi - h);
    return r;
}

__device__ __forceinline__ df2 df_neg(df2 a) {
    a.hi = -a.hi;
    a.lo = -a.lo;
    return a;
}

__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    df2 r;
    r.hi = p + e;
    r.lo = e - (r.hi - p);
    return r;
}

__device__ __forceinline__ float df_to_float(df2 a) { return a.hi + a.lo; }

}  // namespace afmib
