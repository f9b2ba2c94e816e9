// MAC-grid stencils, Helmholtz operator, CG pieces and reductions.
// Memory-bound (FP32) or FP64-pipe-bound (FP64) single-pass kernels: every
// output element is produced by one thread from neighbours that the L1/L2
// caches supply, so DRAM traffic is one read per input array and one write per
// output array.
#include "dfloat.cuh"
#include "kernels.h"
#include <algorithm>

namespace afmib {

namespace {

constexpr int BX = 32, BY = 8;

inline dim3 grid3(const Dims& d) { return dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz); }
inline dim3 block3() { return dim3(BX, BY, 1); }

#define AFMIB_XYZ                                          \
    const int x = blockIdx.x * BX + threadIdx.x;           \
    const int y = blockIdx.y * BY + threadIdx.y;           \
    const int z = blockIdx.z;                              \
    if (x >= d.nx || y >= d.ny) return;

// ---------------------------------------------------------------------------
// Advection, src/ns/solver.h:142-236. Fluxes on the periodic staggering
//   uu(j) = (u(j)+u(j-x))^2/4        at the cell centre left of face j
//   uv(j) = (u(j)+u(j-y))(v(j)+v(j-x))/4 at the edge (x, y, z+1/2)
//   uw(j) = (u(j)+u(j-z))(w(j)+w(j-x))/4 at the edge (x, y+1/2, z)
//   vw(j) = (v(j)+v(j-z))(w(j)+w(j-y))/4 at the edge (x+1/2, y, z)
// and N = n * (flux differences). In channel mode v plane 0 is the zero wall,
// which makes every wall flux of the reference (uvt, uvb, vwt, vwb = 0; vvb,
// vvt from the one interior face) come out of the same formulas.
// ---------------------------------------------------------------------------
// P2: power-of-two grids, 32-bit shift-composed indices and wraps by masks,
// registers capped for 6 resident blocks (the same arithmetic, so the same
// bits as the general form)
template <typename TI, typename T, bool P2>
__global__ void __launch_bounds__(BX * BY, P2 ? 6 : 4) k_advect(Dims d, T* __restrict__ ua, T* __restrict__ va,
                                                                 T* __restrict__ wa, const TI* __restrict__ ui,
                                                                 const TI* __restrict__ vi, const TI* __restrict__ wi) {
    AFMIB_XYZ
    // loads in the storage type TI, arithmetic in T (FP32 for the mixed form)
    struct Ld {
        const TI* p;
        __device__ T operator[](long long k) const { return T(p[k]); }
    } u{ui}, v{vi}, w{wi};
    const T h = T(0.5), n = T(d.n);
    const Ix2 I(d);
    auto lin = [&](const Dims& dd, int xx, int yy, int zz) -> long long {
        return P2 ? (long long)I.at(xx, yy, zz) : afmib::lin(dd, xx, yy, zz);
    };
    const int xm = P2 ? I.xm(x) : xm1(d, x), xp = P2 ? I.xp(x) : xp1(d, x), ym = P2 ? I.ym(y) : ym1(d, y),
              yp = P2 ? I.yp(y) : yp1(d, y), zm = P2 ? I.zm(z) : zm1(d, z), zp = P2 ? I.zp(z) : zp1(d, z);
    const long long i = lin(d, x, y, z);
    const long long ixm = lin(d, xm, y, z), ixp = lin(d, xp, y, z), iym = lin(d, x, ym, z), iyp = lin(d, x, yp, z),
                    izm = lin(d, x, y, zm), izp = lin(d, x, y, zp);
    const T u0 = u[i], v0 = v[i], w0 = w[i];
    T q, r;
    // shared fluxes at this cell's own corner
    q = h * (u0 + u[iym]); r = h * (v0 + v[ixm]); const T uv0 = q * r;
    q = h * (u[izm] + u0); r = h * (w[ixm] + w0); const T uw0 = q * r;
    q = h * (v[izm] + v0); r = h * (w0 + w[iym]); const T vw0 = q * r;
    // u-momentum
    {
        q = h * (u0 + u[ixm]); const T uu0 = q * q;
        q = h * (u[ixp] + u0); const T uup = q * q;
        q = h * (u[iyp] + u0); r = h * (v[iyp] + v[lin(d, xm, yp, z)]); const T uvp = q * r;
        q = h * (u0 + u[izp]); r = h * (w[lin(d, xm, y, zp)] + w[izp]); const T uwp = q * r;
        ua[i] = n * ((uup - uu0) + (uvp - uv0) + (uwp - uw0));
    }
    // v-momentum (plane 0 is the wall in channel mode)
    if (d.channel && y == 0) {
        va[i] = T(0);
    } else {
        q = h * (u[ixp] + u[lin(d, xp, ym, z)]); r = h * (v[ixp] + v0); const T uvp = q * r;
        q = h * (v0 + v[iym]); const T vv0 = q * q;
        q = h * (v[iyp] + v0); const T vvp = q * q;
        q = h * (v0 + v[izp]); r = h * (w[izp] + w[lin(d, x, ym, zp)]); const T vwp = q * r;
        va[i] = n * ((uvp - uv0) + (vvp - vv0) + (vwp - vw0));
    }
    // w-momentum
    {
        q = h * (u[lin(d, xp, y, zm)] + u[ixp]); r = h * (w[ixp] + w0); const T uwp = q * r;
        q = h * (v[lin(d, x, yp, zm)] + v[iyp]); r = h * (w[iyp] + w0); const T vwp = q * r;
        q = h * (w0 + w[izm]); const T ww0 = q * q;
        q = h * (w[izp] + w0); const T wwp = q * q;
        wa[i] = n * ((uwp - uw0) + (vwp - vw0) + (wwp - ww0));
    }
}

// The mixed form's advection of the FP64 velocity, in FP32 from its pairs of
// floats (h: the nearest float, l: the rest, written by the projection; plane
// 0 of v is the zero wall in channel mode as above). The fluxes are those of
// k_advect, but every flux difference is rewritten without cancellation:
//   q1^2 - q0^2       = (q1 - q0)(q1 + q0)            (uu, vv, ww)
//   A1 B1 - A0 B0     = (A1 - A0) B1 + A0 (B1 - B0)   (uv, uw, vw)
// with the differences of velocities formed from the pairs,
// (h_a - h_b) + (l_a - l_b): h_a - h_b is exact when the two are within a
// factor of two (Sterbenz) and otherwise carries an error relative to
// itself, so each difference is its FP32 rounding. FP32 fluxes subtracted
// directly lose n/k of their digits (the difference of two fluxes one cell
// apart), which over 100 steps at 256^3 left the mixed form's velocity 1.3e-8
// from the FP64 form's; here every term is within a few FP32 roundings of
// itself.
template <bool P2>
__global__ void __launch_bounds__(BX * BY, P2 ? 4 : 3) k_advect_df(Dims d, float* __restrict__ ua,
                                                                   float* __restrict__ va, float* __restrict__ wa,
                                                                   const float* __restrict__ uh,
                                                                   const float* __restrict__ ul,
                                                                   const float* __restrict__ vh,
                                                                   const float* __restrict__ vl,
                                                                   const float* __restrict__ wh,
                                                                   const float* __restrict__ wl) {
    AFMIB_XYZ
    const Ix2 I(d);
    auto lin = [&](int xx, int yy, int zz) -> long long {
        return P2 ? (long long)I.at(xx, yy, zz) : afmib::lin(d, xx, yy, zz);
    };
    const int xm = P2 ? I.xm(x) : xm1(d, x), xp = P2 ? I.xp(x) : xp1(d, x), ym = P2 ? I.ym(y) : ym1(d, y),
              yp = P2 ? I.yp(y) : yp1(d, y), zm = P2 ? I.zm(z) : zm1(d, z), zp = P2 ? I.zp(z) : zp1(d, z);
    const long long i = lin(x, y, z);
    const long long ixm = lin(xm, y, z), ixp = lin(xp, y, z), iym = lin(x, ym, z), iyp = lin(x, yp, z),
                    izm = lin(x, y, zm), izp = lin(x, y, zp);
    // difference and sum of two values of a field from its pairs
    auto D = [](const float* h, const float* l, long long a, long long b) { return (h[a] - h[b]) + (l[a] - l[b]); };
    auto S = [](const float* h, const float* l, long long a, long long b) { return (h[a] + h[b]) + (l[a] + l[b]); };
    // q(+1) + 2 q(0) + q(-1) for the squared fluxes
    auto S3 = [](const float* h, const float* l, long long a, long long c, long long b) {
        return ((h[a] + h[b]) + 2.f * h[c]) + ((l[a] + l[b]) + 2.f * l[c]);
    };
    const float f = 0.25f * float(d.n);
    // u-momentum: uu, uv (y), uw (z)
    {
        const long long ixmyp = lin(xm, yp, z), ixmzp = lin(xm, y, zp);
        const float tx = S3(uh, ul, ixp, i, ixm) * D(uh, ul, ixp, ixm);
        const float ty = D(uh, ul, iyp, iym) * S(vh, vl, iyp, ixmyp) +
                         S(uh, ul, i, iym) * (D(vh, vl, iyp, i) + D(vh, vl, ixmyp, ixm));
        const float tz = D(uh, ul, izp, izm) * S(wh, wl, ixmzp, izp) +
                         S(uh, ul, izm, i) * (D(wh, wl, ixmzp, ixm) + D(wh, wl, izp, i));
        ua[i] = f * ((tx + ty) + tz);
    }
    // v-momentum: uv (x), vv, vw (z)
    if (d.channel && y == 0) {
        va[i] = 0.f;
    } else {
        const long long ixpym = lin(xp, ym, z), iymzp = lin(x, ym, zp);
        const float tx = (D(uh, ul, ixp, i) + D(uh, ul, ixpym, iym)) * S(vh, vl, ixp, i) +
                         S(uh, ul, i, iym) * D(vh, vl, ixp, ixm);
        const float ty = S3(vh, vl, iyp, i, iym) * D(vh, vl, iyp, iym);
        const float tz = D(vh, vl, izp, izm) * S(wh, wl, izp, iymzp) +
                         S(vh, vl, izm, i) * (D(wh, wl, izp, i) + D(wh, wl, iymzp, iym));
        va[i] = f * ((tx + ty) + tz);
    }
    // w-momentum: uw (x), vw (y), ww
    {
        const long long ixpzm = lin(xp, y, zm), iypzm = lin(x, yp, zm);
        const float tx = (D(uh, ul, ixpzm, izm) + D(uh, ul, ixp, i)) * S(wh, wl, ixp, i) +
                         S(uh, ul, izm, i) * D(wh, wl, ixp, ixm);
        const float ty = (D(vh, vl, iypzm, izm) + D(vh, vl, iyp, i)) * S(wh, wl, iyp, i) +
                         S(vh, vl, izm, i) * D(wh, wl, iyp, iym);
        const float tz = S3(wh, wl, izp, i, izm) * D(wh, wl, izp, izm);
        wa[i] = f * ((tx + ty) + tz);
    }
}

// Divergence, src/alg/div.h:29-60.
template <typename T>
__global__ void k_div(Dims d, T* __restrict__ out, const T* __restrict__ u, const T* __restrict__ v,
                      const T* __restrict__ w, const T* __restrict__ top, const T* __restrict__ bottom) {
    AFMIB_XYZ
    const long long i = lin(d, x, y, z);
    T dv;
    if (d.channel) {
        const long long ixz = x + (long long)d.nx * z;
        const T tv = top ? top[ixz] : T(0), bv = bottom ? bottom[ixz] : T(0);
        if (d.ny == 1) dv = tv - bv;
        else if (y == 0) dv = v[lin(d, x, 1, z)] - bv;
        else if (y == d.ny - 1) dv = tv - v[i];
        else dv = v[lin(d, x, y + 1, z)] - v[i];
    } else {
        dv = v[lin(d, x, yp1(d, y), z)] - v[i];
    }
    out[i] = T(d.n) * ((u[lin(d, xp1(d, x), y, z)] - u[i]) + dv + (w[lin(d, x, y, zp1(d, z))] - w[i]));
}

// Mixed form: k_div in double-float on the FP32 pipe (GB300's FP64 pipe
// bounds the FP64 kernel: 81% busy, ncu). The FP64 face velocities are split
// by integer operations (df_split, 2^-46 relative), the differences and sums
// are pairs in k_div's order, and the value goes back to FP64 with one
// addition. out_sum[0]: the sum of the written values (the pressure solve's
// mean removal), each thread's pair sum reduced in a fixed order.
__global__ void __launch_bounds__(kRedBlock) k_div_df(Dims d, double* __restrict__ out, const double* __restrict__ u,
                                                     const double* __restrict__ v, const double* __restrict__ w,
                                                     const double* __restrict__ top,
                                                     const double* __restrict__ bottom, RedScratch sc,
                                                     double* out_sum) {
    const int x = blockIdx.x * kRBX + threadIdx.x, y = blockIdx.y * kRBY + threadIdx.y;
    const df2 nn = {float(d.n), 0.f};
    const df2 zero = {0.f, 0.f};
    df2 acc = zero;
    if (x < d.nx && y < d.ny)
        for (int z = blockIdx.z; z < d.nz; z += gridDim.z) {
            const long long i = lin(d, x, y, z);
            df2 dv;
            if (d.channel) {
                const long long ixz = x + (long long)d.nx * z;
                const df2 tv = top ? df_split(top[ixz]) : zero, bv = bottom ? df_split(bottom[ixz]) : zero;
                if (d.ny == 1) dv = df_add(tv, df_neg(bv));
                else if (y == 0) dv = df_add(df_split(v[lin(d, x, 1, z)]), df_neg(bv));
                else if (y == d.ny - 1) dv = df_add(tv, df_neg(df_split(v[i])));
                else dv = df_add(df_split(v[lin(d, x, y + 1, z)]), df_neg(df_split(v[i])));
            } else {
                dv = df_add(df_split(v[lin(d, x, yp1(d, y), z)]), df_neg(df_split(v[i])));
            }
            const df2 du = df_add(df_split(u[lin(d, xp1(d, x), y, z)]), df_neg(df_split(u[i])));
            const df2 dw = df_add(df_split(w[lin(d, x, y, zp1(d, z))]), df_neg(df_split(w[i])));
            const df2 r = df_mul(nn, df_add(df_add(du, dv), dw));
            out[i] = f32_to_f64(r.hi) + f32_to_f64(r.lo);
            acc = df_add(acc, r);
        }
    double a[1] = {f32_to_f64(acc.hi) + f32_to_f64(acc.lo)};
    grid_sum<1>(a, sc, out_sum);
}

// Gradient, src/alg/grad.h:29-44.
template <typename T>
__global__ void k_grad(Dims d, T* __restrict__ px, T* __restrict__ py, T* __restrict__ pz, const T* __restrict__ p) {
    AFMIB_XYZ
    const long long i = lin(d, x, y, z);
    const T n = T(d.n), p0 = p[i];
    px[i] = n * (p0 - p[lin(d, xm1(d, x), y, z)]);
    pz[i] = n * (p0 - p[lin(d, x, y, zm1(d, z))]);
    if (!d.channel || y > 0) py[i] = n * (p0 - p[lin(d, x, ym1(d, y), z)]);
}

// u -= grad(phi), src/ns/projection.h:69-72, saving the wall-adjacent rows that
// the next wall update reads (src/ns/projection.h:91-94).
template <typename T>
__global__ void k_grad_sub(Dims d, T* __restrict__ u, T* __restrict__ v, T* __restrict__ w, const T* __restrict__ p,
                           T* __restrict__ wg, float* __restrict__ u32, float* __restrict__ v32,
                           float* __restrict__ w32, int round_shadow, float* __restrict__ u32l,
                           float* __restrict__ v32l, float* __restrict__ w32l) {
    AFMIB_XYZ
    const long long i = lin(d, x, y, z);
    const T n = T(d.n), p0 = p[i];
    const T gx = n * (p0 - p[lin(d, xm1(d, x), y, z)]);
    const T gz = n * (p0 - p[lin(d, x, y, zm1(d, z))]);
    const T un = u[i] - gx, wn = w[i] - gz;
    u[i] = un;
    w[i] = wn;
    T vn = v[i];
    if (!d.channel || y > 0) {
        vn = vn - n * (p0 - p[lin(d, x, ym1(d, y), z)]);
        v[i] = vn;
    }
    if (u32) {  // FP32 shadow of the velocity for the mixed form's FP32 stencils
        // rounded (or truncated) by integer operations, not by the FP64
        // pipe's conversion
        if constexpr (sizeof(T) == sizeof(double)) {
            if (u32l) {  // the pairs of the mixed form's advection
                const df2 pu = df_split_round(un), pv = df_split_round(vn), pw = df_split_round(wn);
                u32[i] = pu.hi;
                v32[i] = pv.hi;
                w32[i] = pw.hi;
                u32l[i] = pu.lo;
                v32l[i] = pv.lo;
                w32l[i] = pw.lo;
            } else {
                u32[i] = round_shadow ? df_round(un) : df_hi(un);
                v32[i] = round_shadow ? df_round(vn) : df_hi(vn);
                w32[i] = round_shadow ? df_round(wn) : df_hi(wn);
            }
        } else {
            u32[i] = float(un);
            v32[i] = float(vn);
            w32[i] = float(wn);
        }
    }
    if (d.channel && wg) {
        const long long nxz = (long long)d.nx * d.nz, ixz = x + (long long)d.nx * z;
        if (y == 0) { wg[0 * nxz + ixz] = gx; wg[4 * nxz + ixz] = gz; }
        if (y == 1) { wg[1 * nxz + ixz] = gx; wg[6 * nxz + ixz] = gz; }
        if (y == d.ny - 1) { wg[2 * nxz + ixz] = gx; wg[5 * nxz + ixz] = gz; }
        if (y == d.ny - 2) { wg[3 * nxz + ixz] = gx; wg[7 * nxz + ixz] = gz; }
    }
}

// src/ns/projection.h:86-104, including its slips: the loop covers
// nx*min(ny, nz) wall entries and the w corrections read the x-gradient rows.
// corrected: every nx*nz entry, the w corrections from the z-gradient rows.
__global__ void k_wall_update(Dims d, double* __restrict__ walls, const double* __restrict__ wg, int corrected) {
    const long long nxz = (long long)d.nx * d.nz;
    const long long cnt = corrected ? nxz : (long long)d.nx * (d.ny < d.nz ? d.ny : d.nz);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
        const double pxb1 = wg[0 * nxz + i], pxb2 = wg[1 * nxz + i], pxt1 = wg[2 * nxz + i], pxt2 = wg[3 * nxz + i];
        const double pzb1 = wg[4 * nxz + i], pzt1 = wg[5 * nxz + i];
        walls[0 * nxz + i] += (9 * pxt1 - pxt2) / 8;   // ut
        walls[1 * nxz + i] += (9 * pxb1 - pxb2) / 8;   // ub
        const double pzt2 = corrected ? wg[7 * nxz + i] : pxt2;  // the reference reads phidtx here
        const double pzb2 = corrected ? wg[6 * nxz + i] : pxb2;
        walls[2 * nxz + i] += (9 * pzt1 - pzt2) / 8;   // wt
        walls[3 * nxz + i] += (9 * pzb1 - pzb2) / 8;   // wb
    }
}

// (I + s Delta) applied at one point. Cell rows (u, w; all components in
// periodic mode) carry the one-sided Dirichlet closure at the channel walls,
// src/ns/helmholtz.h:90-104; v rows in channel mode treat the walls as zero
// neighbours (plane 0 and its periodic image), src/ns/helmholtz.h:247-248.
template <typename T, typename Get>
__device__ __forceinline__ T helm_point_at(const Dims& d, int comp, T s, Get x, int xi, int yi, int zi) {
    const long long i = lin(d, xi, yi, zi);
    const T off = s * T(d.n) * T(d.n);
    const T x0 = x(i);
    const T sx = x(lin(d, xm1(d, xi), yi, zi)) + x(lin(d, xp1(d, xi), yi, zi));
    if (d.nz == 1) {
        // 2D (periodic): the one-cell z extent folds into the diagonal,
        // src/ns/helmholtz.h:77-88
        const T sy = x(lin(d, xi, ym1(d, yi), zi)) + x(lin(d, xi, yp1(d, yi), zi));
        return (T(1) - T(4) * off) * x0 + off * (sx + sy);
    }
    const T sz = x(lin(d, xi, yi, zm1(d, zi))) + x(lin(d, xi, yi, zp1(d, zi)));
    if (d.channel && comp != 1) {
        T diag = T(1) - T(6) * off;
        T sy;
        if (yi == 0) {
            diag -= T(2) * off;
            sy = (off + off / T(3)) * x(lin(d, xi, 1, zi));
        } else if (yi == d.ny - 1) {
            diag -= T(2) * off;
            sy = (off + off / T(3)) * x(lin(d, xi, yi - 1, zi));
        } else {
            sy = off * (x(lin(d, xi, yi - 1, zi)) + x(lin(d, xi, yi + 1, zi)));
        }
        return diag * x0 + (off * (sx + sz) + sy);
    }
    if (d.channel && comp == 1 && yi == 0) return x0;
    const T sy = x(lin(d, xi, ym1(d, yi), zi)) + x(lin(d, xi, yp1(d, yi), zi));
    return (T(1) - T(6) * off) * x0 + off * (sx + sy + sz);
}

template <typename T>
__device__ __forceinline__ T helm_point(const Dims& d, int comp, T s, const T* __restrict__ x, int xi, int yi, int zi) {
    return helm_point_at(d, comp, s, [x](long long i) { return x[i]; }, xi, yi, zi);
}

template <typename T>
__global__ void k_helm_apply(Dims d, int comp, T s, T* __restrict__ out, const T* __restrict__ in) {
    AFMIB_XYZ
    out[lin(d, x, y, z)] = helm_point(d, comp, s, in, x, y, z);
}

// Right-hand side of the viscous solve, src/ns/solver.h:105-135.
template <typename T, typename TF, typename TA>
__global__ void k_helm_rhs(Dims d, int comp, int be, T* __restrict__ r, const T* __restrict__ uold,
                           const TF* __restrict__ f, const TA* __restrict__ adv, const double* __restrict__ top,
                           const double* __restrict__ bottom, double s_plus, double s_minus, double hdt,
                           double inv_rho) {
    AFMIB_XYZ
    const long long i = lin(d, x, y, z);
    if (d.channel && comp == 1 && y == 0) { r[i] = T(0); return; }
    // wall term of helmholtz_periodic::boundary (u, w rows next to the walls)
    T bm = T(0), bp = T(0);
    const bool wall = d.channel && comp != 1 && (y == 0 || y == d.ny - 1) && top;
    if (wall) {
        const long long ixz = x + (long long)d.nx * z;
        const double wv = (y == 0) ? bottom[ixz] : top[ixz];
        bm = T(8. / 3. * s_minus * d.n * d.n * wv);
        bp = T(8. / 3. * s_plus * d.n * d.n * wv);
    }
    const T src = T(hdt) * (T(inv_rho) * cvt<T, TF>(f[i]) - cvt<T, TA>(adv[i]));
    // away from the wall rows the wall terms are zero and their additions are
    // exact, so they are skipped
    if (be) {
        r[i] = wall ? (uold[i] + T(-1) * bm) + src : uold[i] + src;
    } else {
        const T hp = helm_point(d, comp, T(s_plus), uold, x, y, z);
        r[i] = wall ? (hp + (bp - bm)) + src : hp + src;
    }
}

// Off-diagonal term of the Helmholtz row: helm_point(x) = x0 + off * Q(x) in
// exact arithmetic, with Q = sum(nb) - k x0 (interior, 2D, channel v faces),
// Q = (sx + sz) + 4/3 x(y+-1) - 8 x0 (channel u/w wall rows) and Q = 0 on the
// channel v wall plane (src/ns/helmholtz.h:61-175).
// helm_point (the same expressions, so the same bits) and Q of one cell from
// one set of neighbour loads and partial sums
template <typename T>
__device__ __forceinline__ void helm_point_q(const Dims& d, int comp, T s, const T* __restrict__ x, int xi, int yi,
                                             int zi, T& hx, T& q) {
    const T off = s * T(d.n) * T(d.n);
    const T x0 = x[lin(d, xi, yi, zi)];
    const T sx = x[lin(d, xm1(d, xi), yi, zi)] + x[lin(d, xp1(d, xi), yi, zi)];
    if (d.nz == 1) {
        const T sy = x[lin(d, xi, ym1(d, yi), zi)] + x[lin(d, xi, yp1(d, yi), zi)];
        hx = (T(1) - T(4) * off) * x0 + off * (sx + sy);
        q = (sx + sy) - T(4) * x0;
        return;
    }
    const T sz = x[lin(d, xi, yi, zm1(d, zi))] + x[lin(d, xi, yi, zp1(d, zi))];
    if (d.channel && comp != 1) {
        T diag = T(1) - T(6) * off;
        if (yi == 0 || yi == d.ny - 1) {
            diag -= T(2) * off;
            const T xa = x[lin(d, xi, yi == 0 ? 1 : yi - 1, zi)];
            hx = diag * x0 + (off * (sx + sz) + (off + off / T(3)) * xa);
            q = (sx + sz) + (T(4) / T(3)) * xa - T(8) * x0;
        } else {
            const T sy = x[lin(d, xi, yi - 1, zi)] + x[lin(d, xi, yi + 1, zi)];
            hx = diag * x0 + (off * (sx + sz) + off * sy);
            q = (sx + sz) + sy - T(6) * x0;
        }
        return;
    }
    if (d.channel && comp == 1 && yi == 0) {
        hx = x0;
        q = T(0);
        return;
    }
    const T sy = x[lin(d, xi, ym1(d, yi), zi)] + x[lin(d, xi, yp1(d, yi), zi)];
    const T sum = sx + sy + sz;
    hx = (T(1) - T(6) * off) * x0 + off * sum;
    q = sum - T(6) * x0;
}

// Mixed form, backward-Euler sub-step: the right-hand side b (as k_helm_rhs),
// the first FP64 defect of the viscous solve started from x = uold
// (r = b - H uold, as k_helm_defect, with its squared norm) and Q(uold) for
// the Crank-Nicolson right-hand side of the next sub-step, in one pass.
// DFR (the double-float residual, r_lo given): b is not kept (the later
// residuals are updates) and r = b - H uold is formed as src - bm - off Q,
// equal in exact arithmetic (H x = x + off Q(x) on every row, uold cancels)
// and without uold's cancellation: three FP64 operations fewer per cell.
template <typename TF, typename TA, bool WALK, bool DFR>
__global__ void __launch_bounds__(kRedBlock) k_helm_rhs_be_defect(Dims d, int comp, double* __restrict__ b_out,
                                                                 float* __restrict__ r_out, double* __restrict__ q_out,
                                                                 const double* __restrict__ uold, const TF* __restrict__ f,
                                                                 const TA* __restrict__ adv, const double* __restrict__ top,
                                                                 const double* __restrict__ bottom, double s_minus,
                                                                 double hdt, double inv_rho, RedScratch sc, double* out,
                                                                 float* __restrict__ r_lo, double* __restrict__ uo_out,
                                                                 bool lo_split) {
    float acc = 0.f;
    auto body = [&](int xi, int yi, int zi) {
        const long long i = lin(d, xi, yi, zi);
        double b = 0.0, sb = 0.0;  // b; src - bm (DFR)
        const bool vwall = d.channel && comp == 1 && yi == 0;
        if (!vwall) {
            const double src = hdt * (inv_rho * cvt<double, TF>(f[i]) - cvt<double, TA>(adv[i]));
            if (d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1) && top) {
                const long long ixz = xi + (long long)d.nx * zi;
                const double bm = 8. / 3. * s_minus * d.n * d.n * ((yi == 0) ? bottom[ixz] : top[ixz]);
                if (DFR) sb = src - bm;
                else b = (uold[i] + -1.0 * bm) + src;
            } else {
                if (DFR) sb = src;
                else b = uold[i] + src;
            }
        }
        double hx, q;
        helm_point_q(d, comp, s_minus, uold, xi, yi, zi, hx, q);
        if (!DFR) b_out[i] = b;
        q_out[i] = q;
        if (uo_out) uo_out[i] = uold[i];  // the step's start velocity, kept for the CN sub-step
        const double off = s_minus * double(d.n) * double(d.n);  // helm_point_q's
        const double rd = DFR ? (vwall ? -uold[i] : sb - off * q) : b - hx;
        float lo;
        const float ri = defect_words(rd, r_lo ? &lo : nullptr, lo_split);
        r_out[i] = ri;
        if (r_lo) r_lo[i] = lo;
        acc += ri * ri;
    };
    if (WALK) {
        tile_walk(d, body);
    } else {
        const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
        if (xi < d.nx && yi < d.ny)
            for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) body(xi, yi, zi);
    }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// Mixed form, Crank-Nicolson sub-step: the right-hand side from Q(uold) kept
// by the backward-Euler sub-step, b = (uold + off+ Q + (bp - bm)) + src, a
// pointwise pass instead of the FP64 stencil.
template <typename TF, typename TA>
__global__ void k_helm_rhs_cn_q(Dims d, int comp, double* __restrict__ r, const double* __restrict__ uold,
                                const double* __restrict__ q, const TF* __restrict__ f, const TA* __restrict__ adv,
                                const double* __restrict__ top, const double* __restrict__ bottom, double s_plus,
                                double s_minus, double hdt, double inv_rho) {
    AFMIB_XYZ
    const long long i = lin(d, x, y, z);
    if (d.channel && comp == 1 && y == 0) { r[i] = 0.0; return; }
    const double src = hdt * (inv_rho * cvt<double, TF>(f[i]) - cvt<double, TA>(adv[i]));
    const double off = s_plus * double(d.n) * double(d.n);
    if (d.channel && comp != 1 && (y == 0 || y == d.ny - 1) && top) {
        const long long ixz = x + (long long)d.nx * z;
        const double wv = (y == 0) ? bottom[ixz] : top[ixz];
        const double bm = 8. / 3. * s_minus * d.n * d.n * wv, bp = 8. / 3. * s_plus * d.n * d.n * wv;
        r[i] = ((uold[i] + off * q[i]) + (bp - bm)) + src;
    } else {
        r[i] = (uold[i] + off * q[i]) + src;
    }
}

// Mixed form, Crank-Nicolson sub-step with the double-float residual: the
// viscous solve starts from x = uold instead of the current velocity, so its
// first residual needs no stencil. With b as k_helm_rhs_cn_q forms it and
// H uold = uold + off- Q(uold) (Q kept by the backward-Euler pass),
// r = b - H uold = (off+ - off-) Q + src (+ bp - bm on the channel u/w wall
// rows; -uold on the v wall plane): one FP64 pass at HBM speed. Writes
// x = uold, the residual's double-float pair and out[0] = rh.rh.
template <typename TF, typename TA>
__global__ void __launch_bounds__(kRedBlock) k_helm_cn_first(Dims d, int comp, double* __restrict__ xo,
                                                            float* __restrict__ rh, float* __restrict__ rl,
                                                            const double* __restrict__ uold, const double* __restrict__ q,
                                                            const TF* __restrict__ f, const TA* __restrict__ adv,
                                                            const double* __restrict__ top,
                                                            const double* __restrict__ bottom, double s_plus,
                                                            double s_minus, double hdt, double inv_rho, RedScratch sc,
                                                            double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const double offd = (s_plus - s_minus) * double(d.n) * double(d.n);
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const double u0 = uold[i];
            double rd;
            if (d.channel && comp == 1 && yi == 0) {
                rd = -u0;
            } else {
                double s2 = hdt * (inv_rho * cvt<double, TF>(f[i]) - cvt<double, TA>(adv[i]));
                if (d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1) && top) {
                    const long long ixz = xi + (long long)d.nx * zi;
                    const double wv = (yi == 0) ? bottom[ixz] : top[ixz];
                    const double bm = 8. / 3. * s_minus * d.n * d.n * wv, bp = 8. / 3. * s_plus * d.n * d.n * wv;
                    s2 = s2 + (bp - bm);
                }
                rd = offd * q[i] + s2;
            }
            xo[i] = u0;
            float lo;
            const float hi = defect_words(rd, &lo, true);
            rh[i] = hi;
            rl[i] = lo;
            acc += hi * hi;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// ---------------------------------------------------------------------------
// The two first residuals above without FP64-pipe work (the mixed form's
// default; the FP64 forces case). The FP64 values are split exactly by
// integer operations (df_split, 24 + 23 bits) and the expressions evaluated in
// double-float on the FP32 pipe (df_add, df_mul: relative error a few units
// of 2^-46 of the largest term), with the coefficients handed in as pairs:
//   src = hdt/rho f - hdt adv,
//   BE: r = src (- cbm wall) - off- Q(uold),  Q as helm_point_q,
//   CN: r = offd Q + src (+ cwall wall),      offd = off+ - off-.
// The residual is the double-float pair itself (the FP32 defect the inner
// solve reads is its leading float); Q goes back to FP64 with one addition.
// The first residuals differ from the FP64 passes' by a few units of 2^-46
// of their terms, far below the solver tolerances. Opt-in: in the mixed
// step these passes run on one stream beside the other stream's
// corrections, and taking them off the FP64 pipe measured no faster (56.36
// against 56.49 IB steps/s at 256^3).
// ---------------------------------------------------------------------------
struct DfCoef {
    df2 hdt_rho, hdt, off, cwall, four_thirds;
};

__device__ __forceinline__ df2 dff(float v) {
    df2 r;
    r.hi = v;
    r.lo = 0.f;
    return r;
}
__device__ __forceinline__ df2 df_sub(df2 a, df2 b) { return df_add(a, df_neg(b)); }

// Q(x) of helm_point_q in double-float
__device__ __forceinline__ df2 df_helm_q(const Dims& d, int comp, const double* __restrict__ x, int xi, int yi, int zi,
                                         const DfCoef& c) {
    const df2 x0 = df_split(x[lin(d, xi, yi, zi)]);
    const df2 sx = df_add(df_split(x[lin(d, xm1(d, xi), yi, zi)]), df_split(x[lin(d, xp1(d, xi), yi, zi)]));
    if (d.nz == 1) {
        const df2 sy = df_add(df_split(x[lin(d, xi, ym1(d, yi), zi)]), df_split(x[lin(d, xi, yp1(d, yi), zi)]));
        return df_sub(df_add(sx, sy), df_mul(dff(4.f), x0));
    }
    const df2 sz = df_add(df_split(x[lin(d, xi, yi, zm1(d, zi))]), df_split(x[lin(d, xi, yi, zp1(d, zi))]));
    if (d.channel && comp != 1) {
        if (yi == 0 || yi == d.ny - 1) {
            const df2 xa = df_split(x[lin(d, xi, yi == 0 ? 1 : yi - 1, zi)]);
            return df_sub(df_add(df_add(sx, sz), df_mul(c.four_thirds, xa)), df_mul(dff(8.f), x0));
        }
        const df2 sy = df_add(df_split(x[lin(d, xi, yi - 1, zi)]), df_split(x[lin(d, xi, yi + 1, zi)]));
        return df_sub(df_add(df_add(sx, sz), sy), df_mul(dff(6.f), x0));
    }
    if (d.channel && comp == 1 && yi == 0) return dff(0.f);
    const df2 sy = df_add(df_split(x[lin(d, xi, ym1(d, yi), zi)]), df_split(x[lin(d, xi, yp1(d, yi), zi)]));
    return df_sub(df_add(df_add(sx, sy), sz), df_mul(dff(6.f), x0));
}

template <typename TA>
__device__ __forceinline__ df2 df_src(double f, TA adv, const DfCoef& c) {
    return df_sub(df_mul(c.hdt_rho, df_split(f)), df_mul(c.hdt, df_split((double)adv)));
}

template <typename TA, bool WALK>
__global__ void __launch_bounds__(kRedBlock) k_helm_rhs_be_defect_df(Dims d, int comp, float* __restrict__ r_out,
                                                                    float* __restrict__ r_lo, double* __restrict__ q_out,
                                                                    double* __restrict__ uo_out,
                                                                    const double* __restrict__ uold,
                                                                    const double* __restrict__ f,
                                                                    const TA* __restrict__ adv,
                                                                    const double* __restrict__ top,
                                                                    const double* __restrict__ bottom, DfCoef c,
                                                                    RedScratch sc, double* out) {
    float acc = 0.f;
    auto body = [&](int xi, int yi, int zi) {
        const long long i = lin(d, xi, yi, zi);
        const double u0 = uold[i];
        df2 rd;
        if (d.channel && comp == 1 && yi == 0) {  // the v wall plane
            rd = df_split(-u0);
            q_out[i] = 0.0;
        } else {
            df2 sb = df_src(f[i], adv[i], c);
            if (d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1) && top) {
                const long long ixz = xi + (long long)d.nx * zi;
                sb = df_sub(sb, df_mul(c.cwall, df_split((yi == 0) ? bottom[ixz] : top[ixz])));
            }
            const df2 q = df_helm_q(d, comp, uold, xi, yi, zi, c);
            q_out[i] = f32_to_f64(q.hi) + f32_to_f64(q.lo);
            rd = df_sub(sb, df_mul(c.off, q));
        }
        if (uo_out) uo_out[i] = u0;  // the step's start velocity, kept for the CN sub-step
        r_out[i] = rd.hi;
        r_lo[i] = rd.lo;
        acc += rd.hi * rd.hi;
    };
    if (WALK) {
        tile_walk(d, body);
    } else {
        const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
        if (xi < d.nx && yi < d.ny)
            for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) body(xi, yi, zi);
    }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

template <typename TA>
__global__ void __launch_bounds__(kRedBlock) k_helm_cn_first_df(Dims d, int comp, double* __restrict__ xo,
                                                               float* __restrict__ rh, float* __restrict__ rl,
                                                               const double* __restrict__ uold,
                                                               const double* __restrict__ q,
                                                               const double* __restrict__ f,
                                                               const TA* __restrict__ adv,
                                                               const double* __restrict__ top,
                                                               const double* __restrict__ bottom, DfCoef c,
                                                               RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const double u0 = uold[i];
            df2 rd;
            if (d.channel && comp == 1 && yi == 0) {
                rd = df_split(-u0);
            } else {
                df2 s2 = df_src(f[i], adv[i], c);
                if (d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1) && top) {
                    const long long ixz = xi + (long long)d.nx * zi;
                    s2 = df_add(s2, df_mul(c.cwall, df_split((yi == 0) ? bottom[ixz] : top[ixz])));
                }
                rd = df_add(df_mul(c.off, df_split(q[i])), s2);
            }
            xo[i] = u0;
            rh[i] = rd.hi;
            rl[i] = rd.lo;
            acc += rd.hi * rd.hi;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// ---------------------------------------------------------------------------
// CG pieces. Scalars live on the device in cgs[] = {n0, pq, n1, beta, alpha}
// so that no host round trip sits inside an iteration except the convergence
// test on n0 (the reference's absolute 2-norm stop, src/alg/cg.h:42).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_cg_init(Dims d, int comp, T s, const T* __restrict__ x,
                                                      const T* __restrict__ b, T* __restrict__ r, T* __restrict__ p,
                                                      RedScratch sc, double* cgs) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    T acc = T(0);
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const T ri = b[i] - helm_point(d, comp, s, x, xi, yi, zi);
            r[i] = ri;
            p[i] = ri;
            acc += ri * ri;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, cgs + 0);
}

template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_cg_apply(Dims d, int comp, T s, const T* __restrict__ p,
                                                       T* __restrict__ q, RedScratch sc, double* cgs) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    T acc = T(0);
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const T qi = helm_point(d, comp, s, p, xi, yi, zi);
            q[i] = qi;
            acc += p[i] * qi;
        }
    double a[1] = {(double)acc};
    if (grid_sum<1>(a, sc, cgs + 1)) cgs[4] = cgs[0] / a[0];  // alpha = n0 / (p.Ap)
}

template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_cg_update(long long N, T* __restrict__ x, T* __restrict__ r,
                                                        const T* __restrict__ p, const T* __restrict__ q,
                                                        RedScratch sc, double* cgs) {
    const T alpha = T(cgs[4]);
    T part = T(0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        x[i] = x[i] + alpha * p[i];
        const T ri = r[i] - q[i] * alpha;
        r[i] = ri;
        part += ri * ri;
    }
    double acc[1] = {(double)part};
    if (grid_sum<1>(acc, sc, cgs + 2)) {
        cgs[3] = acc[0] / cgs[0];  // beta = n1 / n0
        cgs[0] = acc[0];
    }
}

// Direction update fused into the next operator apply (FP32 inner solves):
// p' = beta p + r is formed on the fly at the seven stencil points, written
// out of place to pn, and q = H p' with p'.q reduced; alpha in the finisher.
template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_cg_dir_apply(Dims d, int comp, T s, const T* __restrict__ p,
                                                           const T* __restrict__ r, T* __restrict__ pn,
                                                           T* __restrict__ q, RedScratch sc, double* cgs) {
    const T beta = T(cgs[3]);
    auto P = [p, r, beta](long long i) { return p[i] * beta + r[i]; };
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    T acc = T(0);
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const T pi = P(i);
            const T qi = helm_point_at(d, comp, s, P, xi, yi, zi);
            pn[i] = pi;
            q[i] = qi;
            acc += pi * qi;
        }
    double a[1] = {(double)acc};
    if (grid_sum<1>(a, sc, cgs + 1)) cgs[4] = cgs[0] / a[0];
}

template <typename T>
__global__ void k_cg_direction(long long N, T* __restrict__ p, const T* __restrict__ r, const double* cgs) {
    const T beta = T(cgs[3]);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        p[i] = p[i] * beta + r[i];
}

// ---------------------------------------------------------------------------
// Defect-correction pieces of the mixed form: the residual of the FP64 state
// evaluated in FP64 and handed to the FP32 inner solve as an FP32 defect, and
// the FP64 update x += e with the FP32 correction.
// ---------------------------------------------------------------------------
template <typename TD, bool WALK>
__global__ void __launch_bounds__(kRedBlock) k_helm_defect(Dims d, int comp, double s, const double* __restrict__ x,
                                                          const double* __restrict__ b, TD* __restrict__ r,
                                                          RedScratch sc, double* out, float* __restrict__ r_lo,
                                                          bool lo_split) {
    TD acc = TD(0);
    auto body = [&](int xi, int yi, int zi) {
        const long long i = lin(d, xi, yi, zi);
        float lo;
        const TD ri = defect_words(b[i] - helm_point(d, comp, s, x, xi, yi, zi), r_lo ? &lo : nullptr, lo_split);
        r[i] = ri;
        if (r_lo) r_lo[i] = lo;
        acc += ri * ri;
    };
    if (WALK) {
        tile_walk(d, body);
    } else {
        const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
        if (xi < d.nx && yi < d.ny)
#pragma unroll 2
            for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) body(xi, yi, zi);
    }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// The same defect without FP64 instructions: the stencil's FP64 values are
// combined exactly in int64 at the cell's largest exponent and the small
// results are scaled in float pairs (helm_residual_bfp). Rows follow
// helm_point: interior (and 2D, and the channel v faces) H x = x0 + off Q
// with Q = sum(nb) - k x0; channel u/w wall rows H x = x0 + (off/3) Q with
// Q = 3 (sx + sz) + 4 x(y+-1) - 24 x0 (src/ns/helmholtz.h:90-104); the
// channel v wall plane is the identity.
__global__ void __launch_bounds__(kRedBlock) k_helm_defect_bfp(Dims d, int comp, double s, const double* __restrict__ x,
                                                              const double* __restrict__ b, float* __restrict__ r,
                                                              RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const double off = s * (double)d.n * (double)d.n;
    const df2 f1 = df_split(off), f3 = df_split(off / 3.0);
    const int ones[6] = {1, 1, 1, 1, 1, 1}, wallc[5] = {3, 3, 3, 3, 4};
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const double x0 = x[i], bi = b[i];
            double nb[6];
            nb[0] = x[lin(d, xm1(d, xi), yi, zi)];
            nb[1] = x[lin(d, xp1(d, xi), yi, zi)];
            float ri;
            if (d.nz == 1) {
                nb[2] = x[lin(d, xi, ym1(d, yi), zi)];
                nb[3] = x[lin(d, xi, yp1(d, yi), zi)];
                ri = helm_residual_bfp(bi, x0, nb, ones, 4, -4, f1);
            } else {
                nb[2] = x[lin(d, xi, yi, zm1(d, zi))];
                nb[3] = x[lin(d, xi, yi, zp1(d, zi))];
                if (d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1)) {
                    nb[4] = x[lin(d, xi, yi == 0 ? 1 : yi - 1, zi)];
                    ri = helm_residual_bfp(bi, x0, nb, wallc, 5, -24, f3);
                } else if (d.channel && comp == 1 && yi == 0) {
                    ri = helm_residual_bfp(bi, x0, nb, ones, 0, 0, f1);
                } else {
                    nb[4] = x[lin(d, xi, ym1(d, yi), zi)];
                    nb[5] = x[lin(d, xi, yp1(d, yi), zi)];
                    ri = helm_residual_bfp(bi, x0, nb, ones, 6, -6, f1);
                }
            }
            r[i] = ri;
            acc += ri * ri;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// One Jacobi sweep on H x = b (the mixed form's FP32 inner Helmholtz solve):
// x' = x + (b - H x) / diag (as a product with the row's reciprocal), with
// H x from helm_point_at and diag its
// diagonal (1 - 6 off in the interior, 1 - 4 off in 2D, 1 - 8 off on the
// channel u/w wall rows, 1 on the channel v wall plane). x == nullptr starts
// from zero: x' = b / diag.
// helm_point_at with Ix2 indexing (power-of-two extents): same terms, same order
template <typename T>
__device__ __forceinline__ T helm_point2(const Dims& d, const Ix2& I, int comp, T s, const T* __restrict__ x, int xi,
                                         int yi, int zi) {
    const T off = s * T(d.n) * T(d.n);
    const T x0 = x[I.at(xi, yi, zi)];
    const T sx = x[I.at(I.xm(xi), yi, zi)] + x[I.at(I.xp(xi), yi, zi)];
    if (d.nz == 1) {
        const T sy = x[I.at(xi, I.ym(yi), zi)] + x[I.at(xi, I.yp(yi), zi)];
        return (T(1) - T(4) * off) * x0 + off * (sx + sy);
    }
    const T sz = x[I.at(xi, yi, I.zm(zi))] + x[I.at(xi, yi, I.zp(zi))];
    if (d.channel && comp != 1) {
        T diag = T(1) - T(6) * off;
        T sy;
        if (yi == 0) {
            diag -= T(2) * off;
            sy = (off + off / T(3)) * x[I.at(xi, 1, zi)];
        } else if (yi == d.ny - 1) {
            diag -= T(2) * off;
            sy = (off + off / T(3)) * x[I.at(xi, yi - 1, zi)];
        } else {
            sy = off * (x[I.at(xi, yi - 1, zi)] + x[I.at(xi, yi + 1, zi)]);
        }
        return diag * x0 + (off * (sx + sz) + sy);
    }
    if (d.channel && comp == 1 && yi == 0) return x0;
    const T sy = x[I.at(xi, I.ym(yi), zi)] + x[I.at(xi, I.yp(yi), zi)];
    return (T(1) - T(6) * off) * x0 + off * (sx + sy + sz);
}

template <typename T>
__device__ __forceinline__ T helm_diag(const Dims& d, int comp, T off, int y) {
    if (d.nz == 1) return T(1) - T(4) * off;
    if (d.channel && comp != 1 && (y == 0 || y == d.ny - 1)) return (T(1) - T(6) * off) - T(2) * off;
    if (d.channel && comp == 1 && y == 0) return T(1);
    return T(1) - T(6) * off;
}

// ZU cells along z per thread, all computed before any is stored (the
// sweep is out of place, so this only puts ZU cells' loads in flight at once)
template <typename T, int ZU>
__global__ void k_helm_jacobi(Dims d, int comp, T s, const T* __restrict__ xv, T* __restrict__ xo,
                              const T* __restrict__ b) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z0 = blockIdx.z * ZU;
    if (x >= d.nx || y >= d.ny) return;
    const T off = s * T(d.n) * T(d.n);
    const T rdiag = T(1) / helm_diag(d, comp, off, y);
    T val[ZU];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const long long i = lin(d, x, y, z0 + u);
        if (!xv) {
            val[u] = b[i] * rdiag;
        } else {
            const T hx = helm_point_at(d, comp, s, [xv](long long j) { return xv[j]; }, x, y, z0 + u);
            val[u] = xv[i] + (b[i] - hx) * rdiag;
        }
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) xo[lin(d, x, y, z0 + u)] = val[u];
}

// CG started from zero: r = p = b, n0 = b.b
template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_cg_init_zero(long long N, const T* __restrict__ b, T* __restrict__ x,
                                                           T* __restrict__ r, T* __restrict__ p, RedScratch sc,
                                                           double* cgs) {
    T part = T(0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        const T bi = b[i];
        x[i] = T(0);
        r[i] = bi;
        p[i] = bi;
        part += bi * bi;
    }
    double acc[1] = {(double)part};
    grid_sum<1>(acc, sc, cgs + 0);
}

template <typename TE>
__global__ void k_add_correction(long long N, double* __restrict__ x, const TE* __restrict__ e) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        x[i] = x[i] + cvt<double, TE>(e[i]);
}

// The same, four cells per thread and iteration with 16-byte accesses
// (n4 = N / 4; x and e 16-byte aligned)
__global__ void k_add_correction4(long long n4, double2* __restrict__ x, const float4* __restrict__ e) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
        const float4 c = e[q];
        double2 a = x[2 * q], b = x[2 * q + 1];
        a.x = a.x + cvt<double, float>(c.x);
        a.y = a.y + cvt<double, float>(c.y);
        b.x = b.x + cvt<double, float>(c.z);
        b.y = b.y + cvt<double, float>(c.w);
        x[2 * q] = a;
        x[2 * q + 1] = b;
    }
}

// ---------------------------------------------------------------------------
// reductions and vector ops
// ---------------------------------------------------------------------------
template <typename T, bool SQ>
__global__ void __launch_bounds__(kRedBlock) k_sum(long long N, const T* __restrict__ x, RedScratch sc, double* out) {
    T part = T(0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        const T e = x[i];
        part += SQ ? e * e : e;
    }
    double acc[1] = {(double)part};
    grid_sum<1>(acc, sc, out);
}

template <typename T>
__global__ void k_sub_scalar(long long N, T* __restrict__ x, const double* sum, double scale) {
    const T m = T(sum[0] * scale);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        x[i] = x[i] - m;
}

template <typename T>
__global__ void k_fill(long long N, T* __restrict__ x, T v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        x[i] = v;
}

template <typename T>
__global__ void k_axpy(long long N, T* __restrict__ y, const T* __restrict__ x, T a) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        y[i] = y[i] + a * x[i];
}

template <typename T>
__global__ void k_lincomb(long long N, T* __restrict__ y, T a, const T* __restrict__ x, T b, const T* __restrict__ z) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * z[i];
}

template <typename T>
__global__ void k_scale(long long N, T* __restrict__ x, T a) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        x[i] = a * x[i];
}

template <typename TO, typename TI>
__global__ void k_convert(long long N, TO* __restrict__ o, const TI* __restrict__ in) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        o[i] = (TO)in[i];
}

inline int ew_blocks(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

template <typename TI, typename T>
void launch_advect(const Dims& d, T* ua, T* va, T* wa, const TI* u, const TI* v, const TI* w, cudaStream_t s) {
    if (ix2_ok(d)) k_advect<TI, T, true><<<grid3(d), block3(), 0, s>>>(d, ua, va, wa, u, v, w);
    else k_advect<TI, T, false><<<grid3(d), block3(), 0, s>>>(d, ua, va, wa, u, v, w);
}
void launch_advect_df(const Dims& d, float* ua, float* va, float* wa, const float* uh, const float* ul,
                      const float* vh, const float* vl, const float* wh, const float* wl, cudaStream_t s) {
    if (ix2_ok(d)) k_advect_df<true><<<grid3(d), block3(), 0, s>>>(d, ua, va, wa, uh, ul, vh, vl, wh, wl);
    else k_advect_df<false><<<grid3(d), block3(), 0, s>>>(d, ua, va, wa, uh, ul, vh, vl, wh, wl);
}
template <typename T>
void launch_div(const Dims& d, T* out, const T* u, const T* v, const T* w, const T* top, const T* bottom, cudaStream_t s) {
    k_div<T><<<grid3(d), block3(), 0, s>>>(d, out, u, v, w, top, bottom);
}
void launch_div_df(const Dims& d, double* out, const double* u, const double* v, const double* w, const double* top,
                   const double* bottom, RedScratch sc, double* out_sum, cudaStream_t s) {
    k_div_df<<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, out, u, v, w, top, bottom, sc, out_sum);
}
template <typename T>
void launch_grad(const Dims& d, T* px, T* py, T* pz, const T* p, cudaStream_t s) {
    k_grad<T><<<grid3(d), block3(), 0, s>>>(d, px, py, pz, p);
}
template <typename T>
void launch_grad_sub(const Dims& d, T* u, T* v, T* w, const T* phi, T* wallgrad, cudaStream_t s, float* u32,
                     float* v32, float* w32, int round_shadow, float* u32l, float* v32l, float* w32l) {
    k_grad_sub<T><<<grid3(d), block3(), 0, s>>>(d, u, v, w, phi, wallgrad, u32, v32, w32, round_shadow, u32l, v32l,
                                                w32l);
}
void launch_wall_update(const Dims& d, double* walls, const double* wallgrad, cudaStream_t s, int corrected) {
    k_wall_update<<<ew_blocks((long long)d.nx * d.nz), 256, 0, s>>>(d, walls, wallgrad, corrected);
}
template <typename T, typename TF, typename TA>
void launch_helm_rhs(const Dims& d, int comp, int be, T* r, const T* uold, const TF* f, const TA* adv, const double* top,
                     const double* bottom, double s_plus, double s_minus, double dt, double inv_rho, cudaStream_t s) {
    k_helm_rhs<T, TF, TA><<<grid3(d), block3(), 0, s>>>(d, comp, be, r, uold, f, adv, top, bottom, s_plus, s_minus,
                                                        be ? dt / 2 : dt, inv_rho);
}
template <typename TF, typename TA>
void launch_helm_rhs_be_defect(const Dims& d, int comp, double* b, float* r, double* q, const double* uold,
                               const TF* f, const TA* adv, const double* top, const double* bottom, double s_minus,
                               double dt, double inv_rho, RedScratch sc, double* out, cudaStream_t s, int walk_blocks,
                               float* r_lo, double* uo_out) {
#define AFMIB_BE(WALKV, DFRV, GRID)                                                                          \
    k_helm_rhs_be_defect<TF, TA, WALKV, DFRV><<<GRID, dim3(kRBX, kRBY), 0, s>>>(                             \
        d, comp, b, r, q, uold, f, adv, top, bottom, s_minus, dt / 2, inv_rho, sc, out, r_lo, uo_out, lo_split())
    if (walk_blocks > 0) {
        if (r_lo) AFMIB_BE(true, true, walk_grid(d, walk_blocks));
        else AFMIB_BE(true, false, walk_grid(d, walk_blocks));
    } else {
        if (r_lo) AFMIB_BE(false, true, red_grid3(d.nx, d.ny, d.nz));
        else AFMIB_BE(false, false, red_grid3(d.nx, d.ny, d.nz));
    }
#undef AFMIB_BE
}
// hdt = dt/2 (BE) or dt (CN); off = s n^2 of the sub-step's operator (BE: off-,
// CN: off+ - off-); cwall = 8/3 n^2 times s- (BE) or s+ - s- (CN)
static DfCoef df_coef(const Dims& d, double hdt, double inv_rho, double off, double cwall_s) {
    DfCoef c;
    c.hdt_rho = df_split(hdt * inv_rho);
    c.hdt = df_split(hdt);
    c.off = df_split(off);
    c.cwall = df_split(8. / 3. * cwall_s * d.n * d.n);
    c.four_thirds = df_split(4.0 / 3.0);
    return c;
}

template <typename TA>
void launch_helm_rhs_be_defect_df(const Dims& d, int comp, float* r, float* r_lo, double* q, double* uo_out,
                                  const double* uold, const double* f, const TA* adv, const double* top,
                                  const double* bottom, double s_minus, double dt, double inv_rho, RedScratch sc,
                                  double* out, cudaStream_t s, int walk_blocks) {
    const DfCoef c = df_coef(d, dt / 2, inv_rho, s_minus * double(d.n) * double(d.n), s_minus);
    if (walk_blocks > 0)
        k_helm_rhs_be_defect_df<TA, true><<<walk_grid(d, walk_blocks), dim3(kRBX, kRBY), 0, s>>>(
            d, comp, r, r_lo, q, uo_out, uold, f, adv, top, bottom, c, sc, out);
    else
        k_helm_rhs_be_defect_df<TA, false><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(
            d, comp, r, r_lo, q, uo_out, uold, f, adv, top, bottom, c, sc, out);
}
template <typename TA>
void launch_helm_cn_first_df(const Dims& d, int comp, double* x, float* rh, float* rl, const double* uold,
                             const double* q, const double* f, const TA* adv, const double* top, const double* bottom,
                             double s_plus, double s_minus, double dt, double inv_rho, RedScratch sc, double* out,
                             cudaStream_t s) {
    const DfCoef c = df_coef(d, dt, inv_rho, (s_plus - s_minus) * double(d.n) * double(d.n), s_plus - s_minus);
    k_helm_cn_first_df<TA><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, x, rh, rl, uold, q, f, adv,
                                                                                    top, bottom, c, sc, out);
}
template void launch_helm_rhs_be_defect_df<float>(const Dims&, int, float*, float*, double*, double*, const double*,
                                                  const double*, const float*, const double*, const double*, double,
                                                  double, double, RedScratch, double*, cudaStream_t, int);
template void launch_helm_cn_first_df<float>(const Dims&, int, double*, float*, float*, const double*, const double*,
                                             const double*, const float*, const double*, const double*, double, double,
                                             double, double, RedScratch, double*, cudaStream_t);

template <typename TF, typename TA>
void launch_helm_rhs_cn_q(const Dims& d, int comp, double* r, const double* uold, const double* q, const TF* f,
                          const TA* adv, const double* top, const double* bottom, double s_plus, double s_minus,
                          double dt, double inv_rho, cudaStream_t s) {
    k_helm_rhs_cn_q<TF, TA><<<grid3(d), block3(), 0, s>>>(d, comp, r, uold, q, f, adv, top, bottom, s_plus, s_minus, dt,
                                                          inv_rho);
}
template <typename TF, typename TA>
void launch_helm_cn_first(const Dims& d, int comp, double* x, float* rh, float* rl, const double* uold, const double* q,
                          const TF* f, const TA* adv, const double* top, const double* bottom, double s_plus,
                          double s_minus, double dt, double inv_rho, RedScratch sc, double* out, cudaStream_t s) {
    k_helm_cn_first<TF, TA><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(
        d, comp, x, rh, rl, uold, q, f, adv, top, bottom, s_plus, s_minus, dt, inv_rho, sc, out);
}
template void launch_helm_cn_first<double, float>(const Dims&, int, double*, float*, float*, const double*,
                                                  const double*, const double*, const float*, const double*,
                                                  const double*, double, double, double, double, RedScratch, double*,
                                                  cudaStream_t);
template void launch_helm_cn_first<float, float>(const Dims&, int, double*, float*, float*, const double*,
                                                 const double*, const float*, const float*, const double*,
                                                 const double*, double, double, double, double, RedScratch, double*,
                                                 cudaStream_t);
template void launch_helm_rhs_be_defect<double, float>(const Dims&, int, double*, float*, double*, const double*,
                                                       const double*, const float*, const double*, const double*,
                                                       double, double, double, RedScratch, double*, cudaStream_t, int,
                                                       float*, double*);
template void launch_helm_rhs_be_defect<float, float>(const Dims&, int, double*, float*, double*, const double*,
                                                      const float*, const float*, const double*, const double*, double,
                                                      double, double, RedScratch, double*, cudaStream_t, int, float*,
                                                      double*);
template void launch_helm_rhs_cn_q<double, float>(const Dims&, int, double*, const double*, const double*,
                                                  const double*, const float*, const double*, const double*, double,
                                                  double, double, double, cudaStream_t);
template void launch_helm_rhs_cn_q<float, float>(const Dims&, int, double*, const double*, const double*, const float*,
                                                 const float*, const double*, const double*, double, double, double,
                                                 double, cudaStream_t);

template <typename TD>
void launch_helm_defect(const Dims& d, int comp, double scale, const double* x, const double* b, TD* r, RedScratch sc,
                        double* out, cudaStream_t s, int walk_blocks, float* r_lo) {
    if (walk_blocks > 0)
        k_helm_defect<TD, true><<<walk_grid(d, walk_blocks), dim3(kRBX, kRBY), 0, s>>>(d, comp, scale, x, b, r, sc, out,
                                                                                       r_lo, lo_split());
    else
        k_helm_defect<TD, false><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, scale, x, b, r, sc,
                                                                                            out, r_lo, lo_split());
}

// Mixed form, recursive outer residual of a viscous solve: with the FP32
// correction e of the last inner solve, x += e (FP64, as k_add_correction)
// and the residual, kept as a double-float pair (rh: the FP32 residual the
// inner solve reads, the float nearest to the pair; rl: the rest), loses
// H e evaluated in double-float (df_helm_row); out[0] = rh.rh, as the FP64
// defect's norm. HBM bound: 40 bytes per cell, no FP64 stencil.
__global__ void __launch_bounds__(kRedBlock) k_helm_update_df(Dims d, int comp, df2 off, df2 cxa,
                                                             double* __restrict__ x, const float* __restrict__ e,
                                                             float* __restrict__ rh, float* __restrict__ rl,
                                                             RedScratch sc, double* out) {
    float acc = 0.f;
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    if (xi < d.nx && yi < d.ny)
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const float e0 = e[i];
            float nb[6];
            nb[0] = e[lin(d, xm1(d, xi), yi, zi)];
            nb[1] = e[lin(d, xp1(d, xi), yi, zi)];
            df2 he;
            if (d.nz == 1) {
                nb[2] = e[lin(d, xi, ym1(d, yi), zi)];
                nb[3] = e[lin(d, xi, yp1(d, yi), zi)];
                he = df_helm_row(e0, nb, 4, 4.f, off, 0.f, cxa, false);
            } else if (d.channel && comp == 1 && yi == 0) {
                he.hi = e0;  // the v wall plane: identity rows
                he.lo = 0.f;
            } else {
                nb[2] = e[lin(d, xi, yi, zm1(d, zi))];
                nb[3] = e[lin(d, xi, yi, zp1(d, zi))];
                if (d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1)) {
                    const float xa = e[lin(d, xi, yi == 0 ? 1 : yi - 1, zi)];
                    he = df_helm_row(e0, nb, 4, 8.f, off, xa, cxa, true);
                } else {
                    nb[4] = e[lin(d, xi, ym1(d, yi), zi)];
                    nb[5] = e[lin(d, xi, yp1(d, yi), zi)];
                    he = df_helm_row(e0, nb, 6, 6.f, off, 0.f, cxa, false);
                }
            }
            df2 r;
            r.hi = rh[i];
            r.lo = rl[i];
            r = df_add(r, df_neg(he));
            rh[i] = r.hi;
            rl[i] = r.lo;
            x[i] = x[i] + cvt<double, float>(e0);
            acc += r.hi * r.hi;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// The same for power-of-two grids with nz % ZU == 0: each thread takes ZU
// consecutive z cells of one (x, y) column (the column's e values reused from
// registers, 32-bit shift-composed indices, every load of the batch issued
// before the rows are evaluated), blocks walk z batches in steps of grid.z;
// the same arithmetic per cell, so the same bits.
template <int ZU, int MINB>
__global__ void __launch_bounds__(kRedBlock, MINB) k_helm_update_df2(Dims d, int comp, df2 off, df2 cxa,
                                                              double* __restrict__ x, const float* __restrict__ e,
                                                              float* __restrict__ rh, float* __restrict__ rl,
                                                              RedScratch sc, double* out) {
    const Ix2 I(d);
    float acc = 0.f;
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const bool vwall = d.channel && comp == 1 && yi == 0;
    const bool uwall = d.channel && comp != 1 && (yi == 0 || yi == d.ny - 1);
    // in-plane neighbours: x -+ 1 and y -+ 1 (u/w wall rows: the row away from the wall)
    const int ya = uwall ? (yi == 0 ? 1 : yi - 1) : I.ym(yi), yb = I.yp(yi);
    if (xi < d.nx && yi < d.ny)
        for (int zb = blockIdx.z; zb < d.nz / ZU; zb += gridDim.z) {
            const int z0 = zb * ZU;
            // every load of the batch first (independent, in flight together), then the rows
            float col[ZU + 2], ex0[ZU], ex1[ZU], ey0[ZU], ey1[ZU], h[ZU], l[ZU];
            double xv[ZU];
#pragma unroll
            for (int u = 0; u < ZU + 2; ++u) col[u] = e[I.at(xi, yi, (z0 + u - 1) & I.mz)];  // z0 - 1 .. z0 + ZU
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                const int z = z0 + u, i = I.at(xi, yi, z);
                ex0[u] = e[I.at(I.xm(xi), yi, z)];
                ex1[u] = e[I.at(I.xp(xi), yi, z)];
                ey0[u] = e[I.at(xi, ya, z)];
                ey1[u] = uwall ? 0.f : e[I.at(xi, yb, z)];
                h[u] = rh[i];
                l[u] = rl[i];
                xv[u] = x[i];
            }
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                const int i = I.at(xi, yi, z0 + u);
                const float e0 = col[u + 1];
                df2 he;
                if (vwall) {
                    he.hi = e0;
                    he.lo = 0.f;
                } else {
                    float nb[6] = {ex0[u], ex1[u], col[u], col[u + 2], ey0[u], ey1[u]};
                    he = uwall ? df_helm_row(e0, nb, 4, 8.f, off, ey0[u], cxa, true)
                               : df_helm_row(e0, nb, 6, 6.f, off, 0.f, cxa, false);
                }
                df2 r;
                r.hi = h[u];
                r.lo = l[u];
                r = df_add(r, df_neg(he));
                rh[i] = r.hi;
                rl[i] = r.lo;
                x[i] = xv[u] + cvt<double, float>(e0);
                acc += r.hi * r.hi;
            }
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// AFMIB_UPDATE_DF_GENERIC=1: the general kernel on power-of-two grids too
// (read at every launch, so that a test compares both in one process)
static bool update_df_generic() {
    const char* e = std::getenv("AFMIB_UPDATE_DF_GENERIC");
    return e && e[0] == '1';
}

void launch_helm_update_df(const Dims& d, int comp, double scale, double* x, const float* e, float* rh, float* rl,
                           RedScratch sc, double* out, cudaStream_t s) {
    const double off = scale * double(d.n) * double(d.n);
    const df2 o = df_split(off), c = df_split(off + off / 3.0);
    // two z cells per thread: 46.4 IB steps/s at 256^3 against 46.3 for four
    // and 45.5 for eight (more registers, fewer warps) and 45.5 for the
    // general kernel; registers capped for kUpdateMinBlocks resident blocks
    constexpr int ZU = 2;
    if (d.nz > 1 && d.nz % ZU == 0 && ix2_ok(d) && !update_df_generic()) {
        const int gx = (d.nx + kRBX - 1) / kRBX, gy = (d.ny + kRBY - 1) / kRBY;
        int gz = d.nz / ZU;
        if ((long long)gx * gy * gz > kMaxRedBlocks) gz = std::max(1, kMaxRedBlocks / (gx * gy));
        k_helm_update_df2<ZU, kUpdateMinBlocks><<<dim3(gx, gy, gz), dim3(kRBX, kRBY), 0, s>>>(d, comp, o, c, x, e, rh,
                                                                                             rl, sc, out);
        return;
    }
    k_helm_update_df<<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, o, c, x, e, rh, rl, sc, out);
}
template <typename T>
void launch_cg_init_zero(long long n, const T* b, T* x, T* r, T* p, RedScratch sc, double* cgs, cudaStream_t s) {
    k_cg_init_zero<T><<<red_blocks(n), kRedBlock, 0, s>>>(n, b, x, r, p, sc, cgs);
}
template <typename TE>
void launch_add_correction(long long n, double* x, const TE* e, cudaStream_t s) {
    if (sizeof(TE) == 4 && n % 4 == 0 && ((uintptr_t)x % 16) == 0 && ((uintptr_t)e % 16) == 0) {
        k_add_correction4<<<ew_blocks(n / 4), 256, 0, s>>>(n / 4, reinterpret_cast<double2*>(x),
                                                          reinterpret_cast<const float4*>(e));
        return;
    }
    k_add_correction<TE><<<ew_blocks(n), 256, 0, s>>>(n, x, e);
}
template <typename T>
void launch_helm_apply(const Dims& d, int comp, double scale, T* y, const T* x, cudaStream_t s) {
    k_helm_apply<T><<<grid3(d), block3(), 0, s>>>(d, comp, T(scale), y, x);
}
template <typename T>
void launch_cg_init(const Dims& d, int comp, double scale, const T* x, const T* b, T* r, T* p, RedScratch sc,
                    double* cgs, cudaStream_t s) {
    k_cg_init<T><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, T(scale), x, b, r, p, sc, cgs);
}
template <typename T>
void launch_cg_apply(const Dims& d, int comp, double scale, const T* p, T* q, RedScratch sc, double* cgs, cudaStream_t s) {
    k_cg_apply<T><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, T(scale), p, q, sc, cgs);
}
template <typename T, int ZU>
__global__ void k_helm_jacobi2(Dims d, int comp, T s, const T* __restrict__ xv, T* __restrict__ xo,
                               const T* __restrict__ b, int rev) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int x = B.x * BX + threadIdx.x, y = B.y * BY + threadIdx.y, z0 = B.z * ZU;
    if (x >= d.nx || y >= d.ny) return;
    const T off = s * T(d.n) * T(d.n);
    const T rdiag = T(1) / helm_diag(d, comp, off, y);
    T val[ZU];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int i = I.at(x, y, z0 + u);
        val[u] = xv ? xv[i] + (b[i] - helm_point2(d, I, comp, s, xv, x, y, z0 + u)) * rdiag : b[i] * rdiag;
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) xo[I.at(x, y, z0 + u)] = val[u];
}

// One colour of a red-black Gauss-Seidel sweep of the FP32 inner Helmholtz
// solve, in place: x += (b - H x) / diag at the colour's cells (the other
// colour's values are the latest). With init the sweep starts from x = 0: the
// colour's cells take b / diag and the other colour's cells are zeroed. For
// the 7-point operator under red-black ordering the sweep contracts the
// error as the square of the Jacobi rate.
template <typename T, int ZU>
__device__ __forceinline__ void helm_rbgs2_body(Dims d, int comp, T s, int color, int init, T* __restrict__ xv,
                                                const T* __restrict__ b, int rev) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int y = B.y * BY + threadIdx.y, t = B.x * BX + threadIdx.x, z0 = B.z * ZU;
    if (y >= d.ny || 2 * t >= d.nx) return;
    const T off = s * T(d.n) * T(d.n);
    const T rdiag = T(1) / helm_diag(d, comp, off, y);
    T val[ZU];
    int at[ZU];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int z = z0 + u, x = 2 * t + ((y + z + color) & 1);
        const int i = I.at(x, y, z);
        val[u] = init ? b[i] * rdiag : xv[i] + (b[i] - helm_point2(d, I, comp, s, xv, x, y, z)) * rdiag;
        at[u] = i;
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        xv[at[u]] = val[u];
        if (init) xv[I.at(2 * t + ((y + z0 + u + color + 1) & 1), y, z0 + u)] = T(0);
    }
}
template <typename T, int ZU, int MINB>
__global__ void __launch_bounds__(BX * BY, MINB) k_helm_rbgs2b(Dims d, int comp, T s, int color, int init,
                                                              T* __restrict__ xv, const T* __restrict__ b, int rev) {
    helm_rbgs2_body<T, ZU>(d, comp, s, color, init, xv, b, rev);
}

template <typename T>
bool launch_helm_rbgs(const Dims& d, int comp, double scale, int color, int init, T* x, const T* b, cudaStream_t s,
                      int rev) {
    if (!(d.nz % 8 == 0 && d.nx % 2 == 0 && ix2_ok(d))) return false;
    const dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / 8);
    // registers capped for 6 resident blocks (40 against 48): measured with the
    // multigrid smoother's cap, 50.5 against 50.0 IB steps/s at 256^3
    k_helm_rbgs2b<T, 8, 6><<<g, dim3(BX, BY), 0, s>>>(d, comp, T(scale), color, init, x, b, rev);
    return true;
}
template bool launch_helm_rbgs<float>(const Dims&, int, double, int, int, float*, const float*, cudaStream_t, int);

template <typename T>
void launch_helm_jacobi(const Dims& d, int comp, double scale, const T* x, T* xo, const T* b, cudaStream_t s,
                        int rev) {
    const dim3 blk(BX, BY);
    if (d.nz % 8 == 0 && ix2_ok(d))
        k_helm_jacobi2<T, 8><<<dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / 8), blk, 0, s>>>(d, comp, T(scale),
                                                                                                   x, xo, b, rev);
    else if (d.nz % 8 == 0)
        k_helm_jacobi<T, 8><<<dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / 8), blk, 0, s>>>(d, comp, T(scale), x,
                                                                                                  xo, b);
    else
        k_helm_jacobi<T, 1><<<grid3(d), blk, 0, s>>>(d, comp, T(scale), x, xo, b);
}
template void launch_helm_jacobi<float>(const Dims&, int, double, const float*, float*, const float*, cudaStream_t,
                                        int);

template <typename T>
void launch_cg_dir_apply(const Dims& d, int comp, double scale, const T* p, const T* r, T* pn, T* q, RedScratch sc,
                         double* cgs, cudaStream_t s) {
    k_cg_dir_apply<T><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, T(scale), p, r, pn, q, sc, cgs);
}
template <typename T>
void launch_cg_update(long long n, T* x, T* r, const T* p, const T* q, RedScratch sc, double* cgs, cudaStream_t s) {
    k_cg_update<T><<<red_blocks(n), kRedBlock, 0, s>>>(n, x, r, p, q, sc, cgs);
}
template <typename T>
void launch_cg_direction(long long n, T* p, const T* r, const double* cgs, cudaStream_t s) {
    k_cg_direction<T><<<ew_blocks(n), 256, 0, s>>>(n, p, r, cgs);
}
template <typename T>
void launch_sum(long long n, const T* x, RedScratch sc, double* out, cudaStream_t s) {
    k_sum<T, false><<<red_blocks(n), kRedBlock, 0, s>>>(n, x, sc, out);
}
template <typename T>
void launch_sumsq(long long n, const T* x, RedScratch sc, double* out, cudaStream_t s) {
    k_sum<T, true><<<red_blocks(n), kRedBlock, 0, s>>>(n, x, sc, out);
}
template <typename T>
void launch_sub_scalar_scaled(long long n, T* x, const double* sum, double scale, cudaStream_t s) {
    k_sub_scalar<T><<<ew_blocks(n), 256, 0, s>>>(n, x, sum, scale);
}
template <typename T>
void launch_fill(long long n, T* x, T value, cudaStream_t s) {
    k_fill<T><<<ew_blocks(n), 256, 0, s>>>(n, x, value);
}
template <typename T>
void launch_axpy(long long n, T* y, const T* x, T a, cudaStream_t s) {
    k_axpy<T><<<ew_blocks(n), 256, 0, s>>>(n, y, x, a);
}
template <typename T>
void launch_scale(long long n, T* x, T a, cudaStream_t s) {
    k_scale<T><<<ew_blocks(n), 256, 0, s>>>(n, x, a);
}
template <typename T>
void launch_lincomb(long long n, T* y, T a, const T* x, T b, const T* z, cudaStream_t s) {
    k_lincomb<T><<<ew_blocks(n), 256, 0, s>>>(n, y, a, x, b, z);
}
template <typename TO, typename TI>
void launch_convert(long long n, TO* out, const TI* in, cudaStream_t s) {
    k_convert<TO, TI><<<ew_blocks(n), 256, 0, s>>>(n, out, in);
}

// FP32 shadow of an FP64 velocity field (and, with lo, the rest of its
// pair), as k_grad_sub writes it
__global__ void k_shadow(long long N, float* __restrict__ o, const double* __restrict__ in, int round_shadow,
                         float* __restrict__ lo) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        if (lo) {
            const df2 p = df_split_round(in[i]);
            o[i] = p.hi;
            lo[i] = p.lo;
        } else {
            o[i] = round_shadow ? df_round(in[i]) : df_hi(in[i]);
        }
    }
}
void launch_shadow(long long n, float* out, const double* in, cudaStream_t s, int round_shadow, float* lo) {
    k_shadow<<<ew_blocks(n), 256, 0, s>>>(n, out, in, round_shadow, lo);
}

#define AFMIB_INST(T)                                                                                          \
    template void launch_div<T>(const Dims&, T*, const T*, const T*, const T*, const T*, const T*, cudaStream_t); \
    template void launch_grad<T>(const Dims&, T*, T*, T*, const T*, cudaStream_t);                             \
    template void launch_grad_sub<T>(const Dims&, T*, T*, T*, const T*, T*, cudaStream_t, float*, float*, float*, \
                                     int, float*, float*, float*);                                               \
    template void launch_helm_apply<T>(const Dims&, int, double, T*, const T*, cudaStream_t);                  \
    template void launch_cg_init<T>(const Dims&, int, double, const T*, const T*, T*, T*, RedScratch, double*, \
                                    cudaStream_t);                                                             \
    template void launch_cg_apply<T>(const Dims&, int, double, const T*, T*, RedScratch, double*, cudaStream_t); \
    template void launch_cg_update<T>(long long, T*, T*, const T*, const T*, RedScratch, double*, cudaStream_t); \
    template void launch_cg_direction<T>(long long, T*, const T*, const double*, cudaStream_t);                \
    template void launch_sum<T>(long long, const T*, RedScratch, double*, cudaStream_t);                       \
    template void launch_scale<T>(long long, T*, T, cudaStream_t);                                          \
    template void launch_sumsq<T>(long long, const T*, RedScratch, double*, cudaStream_t);                     \
    template void launch_sub_scalar_scaled<T>(long long, T*, const double*, double, cudaStream_t);             \
    template void launch_fill<T>(long long, T*, T, cudaStream_t);                                              \
    template void launch_axpy<T>(long long, T*, const T*, T, cudaStream_t);                                    \
    template void launch_lincomb<T>(long long, T*, T, const T*, T, const T*, cudaStream_t);

AFMIB_INST(double)
AFMIB_INST(float)
template void launch_advect<double, double>(const Dims&, double*, double*, double*, const double*, const double*,
                                            const double*, cudaStream_t);
template void launch_advect<double, float>(const Dims&, float*, float*, float*, const double*, const double*,
                                           const double*, cudaStream_t);
template void launch_advect<float, float>(const Dims&, float*, float*, float*, const float*, const float*,
                                          const float*, cudaStream_t);
template void launch_helm_rhs<double, double, double>(const Dims&, int, int, double*, const double*, const double*,
                                                      const double*, const double*, const double*, double, double,
                                                      double, double, cudaStream_t);
template void launch_helm_rhs<double, float, float>(const Dims&, int, int, double*, const double*, const float*,
                                                    const float*, const double*, const double*, double, double,
                                                    double, double, cudaStream_t);
template void launch_helm_rhs<double, double, float>(const Dims&, int, int, double*, const double*, const double*,
                                                     const float*, const double*, const double*, double, double,
                                                     double, double, cudaStream_t);
void launch_helm_defect_bfp(const Dims& d, int comp, double scale, const double* x, const double* b, float* r,
                            RedScratch sc, double* out, cudaStream_t s) {
    k_helm_defect_bfp<<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, comp, scale, x, b, r, sc, out);
}
template void launch_helm_defect<float>(const Dims&, int, double, const double*, const double*, float*, RedScratch,
                                        double*, cudaStream_t, int, float*);
template void launch_cg_dir_apply<float>(const Dims&, int, double, const float*, const float*, float*, float*,
                                         RedScratch, double*, cudaStream_t);
template void launch_cg_init_zero<float>(long long, const float*, float*, float*, float*, RedScratch, double*,
                                         cudaStream_t);
template void launch_add_correction<float>(long long, double*, const float*, cudaStream_t);
template void launch_convert<float, double>(long long, float*, const double*, cudaStream_t);
template void launch_convert<double, float>(long long, double*, const float*, cudaStream_t);

}  // namespace afmib
