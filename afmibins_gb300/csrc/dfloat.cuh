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

#include <cstdint>
#include <cstring>

namespace afmib {

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ long long dbits(double d) { return __double_as_longlong(d); }
__device__ __forceinline__ double dfrom(unsigned long long u) { return __longlong_as_double((long long)u); }
__device__ __forceinline__ float fbits(unsigned u) { return __int_as_float((int)u); }
__device__ __forceinline__ unsigned fword(float f) { return (unsigned)__float_as_int(f); }
__device__ __forceinline__ int clz64(unsigned long long v) { return __clzll((long long)v); }
#else
inline long long dbits(double d) { long long u; std::memcpy(&u, &d, 8); return u; }
inline double dfrom(unsigned long long u) { double d; std::memcpy(&d, &u, 8); return d; }
inline float fbits(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
inline unsigned fword(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
inline int clz64(unsigned long long v) { return v ? __builtin_clzll(v) : 64; }
#endif
#define AFMIB_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------------------
// FP32 -> FP64 by integer operations (exact, as the IEEE conversion). In the
// mixed form's FP64 kernels that widen FP32 operands (the viscous right-hand
// side, the FP64 += FP32 correction) this measured faster on GB300 than the
// hardware conversion (right-hand side 4.27 -> 4.10 ms per two 256^3 steps);
// the narrowing direction did not (an integer FP64 -> FP32 rounding made the
// FP64 defect kernels 9% slower), so it stays the hardware conversion.
// Zero takes the sign path; subnormal, inf and nan the plain conversion.
// ---------------------------------------------------------------------------
AFMIB_HD double f32_to_f64(float f) {
    const unsigned u = fword(f);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if ((u & 0x7fffffffu) == 0u) return dfrom(sign);  // +-0
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex == 0u || ex == 255u) return (double)f;  // subnormal, inf, nan
    return dfrom(sign | ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29));
}

// TI -> TO, FP32 -> FP64 by f32_to_f64
template <typename TO, typename TI>
AFMIB_HD TO cvt(TI v) { return TO(v); }
template <>
AFMIB_HD double cvt<double, float>(float v) { return f32_to_f64(v); }

struct df2 {
    float hi, lo;
};

// hi = the top 24 significant bits of d (truncated), lo = the next 23, both
// with d's sign; |d| < 2^-126 (float subnormal range and zero) gives 0, and
// lo is dropped below 2^-80. No FP64 instruction is issued.
AFMIB_HD df2 df_split(double d) {
    const unsigned long long u = (unsigned long long)dbits(d);
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
        r.hi = fbits(sign | 0x7f800000u | (mh ? 0x400000u : 0u));
        r.lo = 0.f;
        return r;
    }
    r.hi = fbits(sign | ((unsigned)(e + 127) << 23) | mh);
    const int el = e - 46;  // lo = ml * 2^(e - 46)
    if (el < -126 || ml == 0u) {
        r.lo = 0.f;
        return r;
    }
    const float m = fbits(0x4B000000u | ml) - 8388608.0f;  // ml as a float, exactly
    const float sc = fbits((unsigned)(el + 127) << 23);     // 2^el
    r.lo = fbits(fword(m * sc) | sign);
    return r;
}

// The first word of df_split alone: the float of d's top 24 significant
// bits (truncated toward zero), by integer operations; 0 below the float
// normal range, inf or nan beyond it. On GB300 the hardware FP64 -> FP32
// conversion takes an FP64-pipe slot.
AFMIB_HD float df_hi(double d) {
    const unsigned long long u = (unsigned long long)dbits(d);
    const unsigned hw = (unsigned)(u >> 32), lw = (unsigned)u;
    const unsigned sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7ffu) - 1023;
    const unsigned mh = ((hw & 0xfffffu) << 3) | (lw >> 29);
    if (e < -126) return fbits(sign);
    if (e > 127) return fbits(sign | 0x7f800000u | (mh ? 0x400000u : 0u));
    return fbits(sign | ((unsigned)(e + 127) << 23) | mh);
}

// The float nearest to d (ties away from zero), by integer operations: half
// of the 29 dropped mantissa bits is added to d's bit pattern (a carry moves
// into the exponent, which is the rounding up to the next binade) and the
// result truncated as df_hi. inf and nan pass through df_hi unchanged.
AFMIB_HD float df_round(double d) {
    const unsigned long long u = (unsigned long long)dbits(d);
    if (((u >> 52) & 0x7ffu) == 0x7ffu) return df_hi(d);
    return df_hi(dfrom(u + (1ull << 28)));
}

// d as the float nearest to it (df_round) and the float of the rest: the
// truncated pair of df_split gives the rest exactly, lo - (hi - hi_trunc)
// (both multiples of d's 2^-46 unit below one ulp of hi), so hi + lo is d
// to 2^-46 relative, as df_split's pair. No FP64 instruction is issued.
// Below 2^-80 df_split drops the rest (float underflow): there the
// truncated pair is returned.
AFMIB_HD df2 df_split_round(double d) {
    const df2 t = df_split(d);
    if (t.lo == 0.f) return t;  // no rest, or below the rest's float range
    df2 r;
    r.hi = df_round(d);
    r.lo = t.lo - (r.hi - t.hi);
    return r;
}

// a + b with both pairs' rounding errors carried (accurate under cancellation)
AFMIB_HD df2 df_add(df2 a, df2 b) {
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

AFMIB_HD df2 df_neg(df2 a) {
    a.hi = -a.hi;
    a.lo = -a.lo;
    return a;
}

AFMIB_HD df2 df_mul(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    df2 r;
    r.hi = p + e;
    r.lo = e - (r.hi - p);
    return r;
}

AFMIB_HD float df_to_float(df2 a) { return a.hi + a.lo; }

// sin(pi x) and cos(pi x) for 0 <= x <= 1/2, x and the results as pairs
// (relative error a few units of 2^-46): x > 1/4 is reflected to 1/2 - x
// (sine and cosine swap), theta = pi y <= pi/4, and the Taylor series
//   sin theta = theta (1 - theta^2/(2*3) (1 - theta^2/(4*5) (... (1 - theta^2/(14*15)))))
//   cos theta = 1 - theta^2/(1*2) (1 - theta^2/(3*4) (... (1 - theta^2/(15*16))))
// run to theta^15 and theta^16 (the first terms left out are below 5e-17 of
// the result), evaluated inside out in pair arithmetic. The constants are pi
// and the 1/(k (k+1)) split into float pairs (hi the nearest float, lo the
// nearest float to the rest).
AFMIB_HD void df_sincospi(df2 x, df2* sp, df2* cp) {
    const df2 one = {1.f, 0.f};
    const bool refl = x.hi > 0.25f;
    const df2 half = {0.5f, 0.f};
    const df2 y = refl ? df_add(half, df_neg(x)) : x;
    const df2 pi = {0x1.921fb6p+1f, -0x1.777a5cp-24f};
    const df2 th = df_mul(pi, y);
    const df2 t2 = df_mul(th, th);
    const df2 cs[7] = {{0x1.555556p-3f, -0x1.555556p-28f}, {0x1.99999ap-5f, -0x1.99999ap-31f},
                       {0x1.861862p-6f, -0x1.e79e7ap-32f}, {0x1.c71c72p-7f, -0x1.c71c72p-34f},
                       {0x1.29e412p-7f, 0x1.3c8254p-32f},  {0x1.a41a42p-8f, -0x1.6f96fap-34f},
                       {0x1.381382p-8f, -0x1.8fd8fep-33f}};  // 1/6, 1/20, 1/42, 1/72, 1/110, 1/156, 1/210
    const df2 cc[8] = {{0x1p-1f, 0.f},                      {0x1.555556p-4f, -0x1.555556p-29f},
                       {0x1.111112p-5f, -0x1.dddddep-30f}, {0x1.24924ap-6f, -0x1.b6db6ep-31f},
                       {0x1.6c16c2p-7f, -0x1.27d27ep-32f}, {0x1.f07c2p-8f, -0x1.f07c2p-33f},
                       {0x1.681682p-8f, -0x1.2fd2fep-33f}, {0x1.111112p-8f, -0x1.dddddep-33f}};  // 1/2 .. 1/240
    df2 ts = one, tc = one;
    for (int k = 6; k >= 0; --k) ts = df_add(one, df_neg(df_mul(df_mul(t2, cs[k]), ts)));
    for (int k = 7; k >= 0; --k) tc = df_add(one, df_neg(df_mul(df_mul(t2, cc[k]), tc)));
    const df2 sn = df_mul(th, ts);
    *sp = refl ? tc : sn;
    *cp = refl ? sn : tc;
}

// An FP64 residual as the FP32 defect of the inner solves and, when rest is
// given, the rest of its double-float pair. split: by integer operations
// (df_split: the top 24 bits truncated, the next 23 bits), no FP64-pipe
// instruction; else the hardware rounding and the rounded exact difference.
AFMIB_HD float defect_words(double rd, float* rest, bool split) {
    if (!rest) return (float)rd;
    if (split) {
        const df2 p = df_split(rd);
        *rest = p.lo;
        return p.hi;
    }
    const float h = (float)rd;
    *rest = (float)(rd - f32_to_f64(h));
    return h;
}

// a + b as an exact pair (Knuth's two-sum)
AFMIB_HD df2 two_sum_f(float a, float b) {
    df2 r;
    r.hi = a + b;
    const float v = r.hi - a;
    r.lo = (a - (r.hi - v)) + (b - v);
    return r;
}

// a + b for a pair and a float, renormalised
AFMIB_HD df2 df_add_f(df2 a, float b) {
    df2 s = two_sum_f(a.hi, b);
    s.lo += a.lo;
    df2 r;
    r.hi = s.hi + s.lo;
    r.lo = s.lo - (r.hi - s.hi);
    return r;
}

// One row of the pressure Laplacian applied to an FP32 correction e, in
// double-float: L e = off (sum(nb) - c e0), off = n^2 (exact as a float for
// n < 4096; missing channel neighbours passed as 0).
AFMIB_HD df2 df_lap_row(float e0, const float* nb, int nnb, float c, float off) {
    df2 q;
    q.hi = nb[0];
    q.lo = 0.f;
    for (int j = 1; j < nnb; ++j) q = df_add_f(q, nb[j]);
    df2 ce;
    ce.hi = c * e0;
    ce.lo = fmaf(c, e0, -ce.hi);
    q = df_add(q, df_neg(ce));
    df2 o;
    o.hi = off;
    o.lo = 0.f;
    return df_mul(q, o);
}

// ---------------------------------------------------------------------------
// One row of the viscous operator applied to an FP32 correction e, in
// double-float: H e = e0 + off Q(e), Q = sum(nb) - k e0, plus cxa * xa for
// the channel u/w wall rows (there nb are the x and z neighbours, k = 8, xa
// the neighbour away from the wall and cxa = off + off/3; the FP64 rows are
// helm_point's). The neighbour sum, k e0 (an exact product by fma) and the
// two coefficient products are carried as pairs, so H e has a relative error
// of a few units of 2^-46 of its largest term: the mixed form subtracts it
// from the outer residual instead of re-evaluating b - H x in FP64.
// ---------------------------------------------------------------------------
AFMIB_HD df2 df_helm_row(float e0, const float* nb, int nnb, float k, df2 off, float xa, df2 cxa, bool wall) {
    df2 q;
    q.hi = nb[0];
    q.lo = 0.f;
    for (int j = 1; j < nnb; ++j) q = df_add_f(q, nb[j]);
    df2 ke;
    ke.hi = k * e0;
    ke.lo = fmaf(k, e0, -ke.hi);
    q = df_add(q, df_neg(ke));
    df2 h = df_mul(off, q);
    if (wall) {
        df2 a;
        a.hi = xa;
        a.lo = 0.f;
        h = df_add(h, df_mul(cxa, a));
    }
    return df_add_f(h, e0);
}

// ---------------------------------------------------------------------------
// Per-cell block floating point. The FP64 values of one stencil are taken to
// int64 at a common scale set by the largest exponent E among them (biased):
// value = q * 2^(E - 1078), so |q| < 2^56 and sums of up to 64 such terms
// cannot overflow. Sums and differences are then exact; a value smaller than
// the largest by more than 2^56 loses its bits below that resolution, which
// is 2^-55 of the largest value. Results go back to df pairs (48 bits).
// Zero and FP64 subnormals read as zero. No FP64 instruction is issued.
// ---------------------------------------------------------------------------
AFMIB_HD int bexp(double v) { return (int)(((unsigned long long)dbits(v) >> 52) & 0x7ffu); }

AFMIB_HD long long to_fixed(double v, int E) {
    const unsigned long long u = (unsigned long long)dbits(v);
    const int e = (int)((u >> 52) & 0x7ffu);
    if (e == 0) return 0;
    const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = e - E + 3;  // <= 3
    unsigned long long q;
    if (sh >= 0) q = m << sh;
    else if (sh > -64) q = m >> (-sh);
    else q = 0;
    return (u >> 63) ? -(long long)q : (long long)q;
}

// a float with the 24 leading bits of a (a > 0, top bit at position p) times 2^x
AFMIB_HD float lead24(unsigned long long a, int p, int x) {
    const unsigned long long h = p >= 23 ? (a >> (p - 23)) : (a << (23 - p));
    const int fe = p + x + 127;
    if (fe < 1) return 0.f;  // below the float normal range: negligible here
    if (fe > 254) return fbits(0x7f800000u);
    return fbits(((unsigned)fe << 23) | ((unsigned)h & 0x7fffffu));
}

// q * 2^(E - 1078) as a df pair (hi: 24 leading bits, lo: the next 24)
AFMIB_HD df2 from_fixed(long long q, int E) {
    df2 r;
    r.hi = 0.f;
    r.lo = 0.f;
    if (q == 0) return r;
    const bool neg = q < 0;
    const unsigned long long a = neg ? (unsigned long long)(-q) : (unsigned long long)q;
    const int x = E - 1078;
    const int p = 63 - clz64(a);
    r.hi = lead24(a, p, x);
    if (p > 23) {
        const unsigned long long rem = a & ((1ull << (p - 23)) - 1ull);
        if (rem) r.lo = lead24(rem, 63 - clz64(rem), x);
    }
    if (neg) {
        r.hi = -r.hi;
        r.lo = -r.lo;
    }
    return r;
}

// v * 2^-k by exponent arithmetic (exact; 0 below the FP64 normal range)
AFMIB_HD double scale_pow2_down(double v, int k) {
    long long u = dbits(v);
    const int e = (int)(((unsigned long long)u >> 52) & 0x7ffu);
    if (e == 0 || k == 0) return v;
    if (e - k < 1) return 0.0 * v;
    u -= (long long)k << 52;
    double r;
#if defined(__CUDA_ARCH__)
    r = __longlong_as_double(u);
#else
    std::memcpy(&r, &u, 8);
#endif
    return r;
}

// Mixed-form residual at one cell, r = b - (x0 + f * Q), Q an exact integer
// combination of the stencil values: Q = sum_i cnb[i] * nb[i] + coef0 * x0,
// f the operator's scale as a df pair. Returns r rounded to float.
AFMIB_HD float helm_residual_bfp(double b, double x0, const double* nb, const int* cnb, int nnb, int coef0, df2 f) {
    int E = bexp(b) > bexp(x0) ? bexp(b) : bexp(x0);
    for (int i = 0; i < nnb; ++i) E = bexp(nb[i]) > E ? bexp(nb[i]) : E;
    const long long q0 = to_fixed(x0, E);
    long long Q = (long long)coef0 * q0;
    for (int i = 0; i < nnb; ++i) Q += (long long)cnb[i] * to_fixed(nb[i], E);
    const long long Db = to_fixed(b, E) - q0;
    const df2 r = df_add(from_fixed(Db, E), df_neg(df_mul(f, from_fixed(Q, E))));
    return df_to_float(r);
}

// Laplacian residual r = b - n^2 (sum(nb) - c x0) with n^2 = 2^k2: b is
// brought to the stencil's scale exactly (b 2^-k2), the whole combination
// Q = b 2^-k2 - sum(nb) + c x0 is exact, and r = 2^k2 Q.
AFMIB_HD float lap_residual_bfp(double b, double x0, const double* nb, int nnb, int c, int k2) {
    const double bs = scale_pow2_down(b, k2);
    int E = bexp(bs) > bexp(x0) ? bexp(bs) : bexp(x0);
    for (int i = 0; i < nnb; ++i) E = bexp(nb[i]) > E ? bexp(nb[i]) : E;
    long long Q = to_fixed(bs, E) + (long long)c * to_fixed(x0, E);
    for (int i = 0; i < nnb; ++i) Q -= to_fixed(nb[i], E);
    const df2 q = from_fixed(Q, E);
    const float sc = fbits((unsigned)(k2 + 127) << 23);  // 2^k2, k2 <= 126
    return (q.hi + q.lo) * sc;
}

}  // namespace afmib
