// Geometric multigrid pieces for the pressure projection (src/mg/solver.h,
// src/mg/laplacian.h): red-black Gauss–Seidel in place of the reference's
// lexicographic CSR sweep, the reference's full-weighting restriction and
// trilinear prolongation, and a one-block CG for the coarsest level.
#include <cooperative_groups.h>

#include "dfloat.cuh"
#include "kernels.h"

namespace afmib {

namespace {

constexpr int BX = 32, BY = 8;
inline dim3 grid3(const Dims& d) { return dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz); }

// Neighbour sum and diagonal factor of the Laplacian row at (x, y, z):
// L x = n^2 * (S - c * x_i), c = 6 in the interior and one less per channel
// wall (Neumann, src/mg/laplacian.h:75-82). A one-cell z extent (2D) folds
// its two self-neighbours into the diagonal, src/mg/laplacian.h:62-73.
template <typename T>
__device__ __forceinline__ void lap_row(const Dims& d, const T* x, int xi, int yi, int zi, T& S, T& c) {
    if (d.nz == 1) {
        S = x[lin(d, xm1(d, xi), yi, zi)] + x[lin(d, xp1(d, xi), yi, zi)];
        c = T(4);
    } else {
        S = (x[lin(d, xm1(d, xi), yi, zi)] + x[lin(d, xp1(d, xi), yi, zi)]) +
            (x[lin(d, xi, yi, zm1(d, zi))] + x[lin(d, xi, yi, zp1(d, zi))]);
        c = T(6);
    }
    if (d.channel) {
        if (yi > 0) S += x[lin(d, xi, yi - 1, zi)]; else c -= T(1);
        if (yi < d.ny - 1) S += x[lin(d, xi, yi + 1, zi)]; else c -= T(1);
    } else {
        S += x[lin(d, xi, ym1(d, yi), zi)] + x[lin(d, xi, yp1(d, yi), zi)];
    }
}

template <typename T>
__global__ void k_lap(Dims d, T* __restrict__ out, const T* __restrict__ in) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= d.nx || y >= d.ny) return;
    T S, c;
    lap_row(d, in, x, y, z, S, c);
    const T off = T(d.n) * T(d.n);
    out[lin(d, x, y, z)] = off * (S - c * in[lin(d, x, y, z)]);
}

// r = b - L x at one cell
template <typename T>
__device__ __forceinline__ void residual_cell(const Dims& d, T* r, const T* xv, const T* b, int x, int y, int z) {
    T S, c;
    lap_row(d, xv, x, y, z, S, c);
    const long long i = lin(d, x, y, z);
    const T off = T(d.n) * T(d.n);
    r[i] = b[i] - off * (S - c * xv[i]);
}

template <typename T>
__global__ void k_residual(Dims d, T* __restrict__ r, const T* __restrict__ xv, const T* __restrict__ b) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= d.nx || y >= d.ny) return;
    residual_cell(d, r, xv, b, x, y, z);
}

template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_residual_norm(Dims d, T* __restrict__ r, const T* __restrict__ xv,
                                                            const T* __restrict__ b, RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const T off = T(d.n) * T(d.n);
    T acc = T(0);
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            T S, c;
            lap_row(d, xv, xi, yi, zi, S, c);
            const long long i = lin(d, xi, yi, zi);
            const T ri = b[i] - off * (S - c * xv[i]);
            r[i] = ri;
            acc += ri * ri;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// Mixed form: defect of the FP64 potential, r = b - L x evaluated in FP64 and
// stored in TD for the FP32 inner V-cycles; out[0] = r.r.
// r_lo: also the rest of the FP64 residual, float(r - r_float), the second
// word of the double-float pair that k_lap_update_df updates.
template <typename TD>
__global__ void __launch_bounds__(kRedBlock) k_lap_defect(Dims d, TD* __restrict__ r, const double* __restrict__ xv,
                                                         const double* __restrict__ b, RedScratch sc, double* out,
                                                         float* __restrict__ r_lo, bool lo_split) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const double off = double(d.n) * double(d.n);
    TD acc = TD(0);
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            double S, c;
            lap_row(d, xv, xi, yi, zi, S, c);
            const long long i = lin(d, xi, yi, zi);
            float lo;
            const TD ri = defect_words(b[i] - off * (S - c * xv[i]), r_lo ? &lo : nullptr, lo_split);
            r[i] = ri;
            if (r_lo) r_lo[i] = lo;
            acc += ri * ri;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// Mixed form: the first defect of a pressure solve in double-float on the
// FP32 pipe (the FP64 kernel is FP64-pipe bound: 81% busy, ncu), with the
// mean removal of b folded in: r = (b - m) - n^2 (S - c x0), m = sum * scale
// (the FP64 form's k_sub_scalar value; sum null: m = 0). lap_row's neighbour
// sum in its order, each FP64 value split by integer operations (df_split),
// c x0 and the n^2 scaling as pair products; the pair is the FP32 defect rh
// and its rest rl of k_lap_update_df, out[0] = rh.rh.
__global__ void __launch_bounds__(kRedBlock) k_lap_defect_df(Dims d, float* __restrict__ rh, float* __restrict__ rl,
                                                            const double* __restrict__ xv,
                                                            const double* __restrict__ b, const double* sum,
                                                            double scale, RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const df2 off = {float(d.n) * float(d.n), 0.f};  // exact for n < 4096
    const df2 m = sum ? df_split(sum[0] * scale) : df2{0.f, 0.f};
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            df2 S;
            float c;
            if (d.nz == 1) {
                S = df_add(df_split(xv[lin(d, xm1(d, xi), yi, zi)]), df_split(xv[lin(d, xp1(d, xi), yi, zi)]));
                c = 4.f;
            } else {
                S = df_add(df_add(df_split(xv[lin(d, xm1(d, xi), yi, zi)]), df_split(xv[lin(d, xp1(d, xi), yi, zi)])),
                           df_add(df_split(xv[lin(d, xi, yi, zm1(d, zi))]), df_split(xv[lin(d, xi, yi, zp1(d, zi))])));
                c = 6.f;
            }
            if (d.channel) {
                if (yi > 0) S = df_add(S, df_split(xv[lin(d, xi, yi - 1, zi)])); else c -= 1.f;
                if (yi < d.ny - 1) S = df_add(S, df_split(xv[lin(d, xi, yi + 1, zi)])); else c -= 1.f;
            } else {
                S = df_add(S, df_add(df_split(xv[lin(d, xi, ym1(d, yi), zi)]), df_split(xv[lin(d, xi, yp1(d, yi), zi)])));
            }
            const long long i = lin(d, xi, yi, zi);
            const df2 cx = df_mul(df2{c, 0.f}, df_split(xv[i]));
            const df2 L = df_mul(off, df_add(S, df_neg(cx)));
            const df2 r = df_add(df_add(df_split(b[i]), df_neg(m)), df_neg(L));
            rh[i] = r.hi;
            rl[i] = r.lo;
            acc += r.hi * r.hi;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// Mixed form, recursive outer residual of the pressure solve: with the FP32
// correction e of the inner V-cycles, x += e (FP64) and the residual, kept
// as a double-float pair (rh: the FP32 right-hand side of the V-cycles, rl:
// the rest), loses L e evaluated in double-float (df_lap_row); out[0] =
// rh.rh, as the FP64 defect's norm.
__global__ void __launch_bounds__(kRedBlock) k_lap_update_df(Dims d, double* __restrict__ x,
                                                            const float* __restrict__ e, float* __restrict__ rh,
                                                            float* __restrict__ rl, RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const float off = float(d.n) * float(d.n);
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            const float e0 = e[i];
            float nb[6];
            int m = 0;
            nb[m++] = e[lin(d, xm1(d, xi), yi, zi)];
            nb[m++] = e[lin(d, xp1(d, xi), yi, zi)];
            if (d.nz > 1) {
                nb[m++] = e[lin(d, xi, yi, zm1(d, zi))];
                nb[m++] = e[lin(d, xi, yi, zp1(d, zi))];
            }
            float c = d.nz > 1 ? 6.f : 4.f;
            if (d.channel) {
                if (yi > 0) nb[m++] = e[lin(d, xi, yi - 1, zi)]; else c -= 1.f;
                if (yi < d.ny - 1) nb[m++] = e[lin(d, xi, yi + 1, zi)]; else c -= 1.f;
            } else {
                nb[m++] = e[lin(d, xi, ym1(d, yi), zi)];
                nb[m++] = e[lin(d, xi, yp1(d, yi), zi)];
            }
            for (int j = m; j < 6; ++j) nb[j] = 0.f;
            const df2 le = df_lap_row(e0, nb, 6, c, off);
            df2 r;
            r.hi = rh[i];
            r.lo = rl[i];
            r = df_add(r, df_neg(le));
            rh[i] = r.hi;
            rl[i] = r.lo;
            x[i] = x[i] + cvt<double, float>(e0);
            acc += r.hi * r.hi;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// The same on power-of-two 3D grids, two z cells per thread with every load
// of the pair issued first (as k_helm_update_df2); the same rows, so the
// same bits.
template <int ZU, int MINB>
__global__ void __launch_bounds__(kRedBlock, MINB) k_lap_update_df2(Dims d, double* __restrict__ x,
                                                             const float* __restrict__ e, float* __restrict__ rh,
                                                             float* __restrict__ rl, RedScratch sc, double* out) {
    const Ix2 I(d);
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const float off = float(d.n) * float(d.n);
    const bool has_ym = !d.channel || yi > 0, has_yp = !d.channel || yi < d.ny - 1;
    const float c = 6.f - (has_ym ? 0.f : 1.f) - (has_yp ? 0.f : 1.f);
    const int ym = I.ym(yi), yp = I.yp(yi);
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
        for (int zb = blockIdx.z; zb < d.nz / ZU; zb += gridDim.z) {
            const int z0 = zb * ZU;
            float col[ZU + 2], ex0[ZU], ex1[ZU], ey0[ZU], ey1[ZU], h[ZU], l[ZU];
            double xv[ZU];
#pragma unroll
            for (int u = 0; u < ZU + 2; ++u) col[u] = e[I.at(xi, yi, (z0 + u - 1) & I.mz)];  // z0 - 1 .. z0 + ZU
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                const int z = z0 + u, i = I.at(xi, yi, z);
                ex0[u] = e[I.at(I.xm(xi), yi, z)];
                ex1[u] = e[I.at(I.xp(xi), yi, z)];
                ey0[u] = has_ym ? e[I.at(xi, ym, z)] : 0.f;
                ey1[u] = has_yp ? e[I.at(xi, yp, z)] : 0.f;
                h[u] = rh[i];
                l[u] = rl[i];
                xv[u] = x[i];
            }
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                const int i = I.at(xi, yi, z0 + u);
                const float e0 = col[u + 1];
                // the general kernel's neighbour order: x, z, then the y neighbours present
                float nb[6] = {ex0[u], ex1[u], col[u], col[u + 2], has_ym ? ey0[u] : ey1[u], has_ym ? ey1[u] : 0.f};
                if (!has_yp) nb[5] = 0.f;
                const df2 le = df_lap_row(e0, nb, 6, c, off);
                df2 r;
                r.hi = h[u];
                r.lo = l[u];
                r = df_add(r, df_neg(le));
                rh[i] = r.hi;
                rl[i] = r.lo;
                x[i] = xv[u] + cvt<double, float>(e0);
                acc += r.hi * r.hi;
            }
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// The same defect without FP64 instructions (lap_residual_bfp): with
// n^2 = 2^k2, b 2^-k2 - sum(nb) + c x0 is formed exactly in int64 at the
// cell's largest exponent and scaled back by 2^k2.
__global__ void __launch_bounds__(kRedBlock) k_lap_defect_bfp(Dims d, int k2, float* __restrict__ r,
                                                             const double* __restrict__ xv, const double* __restrict__ b,
                                                             RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    float acc = 0.f;
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            const long long i = lin(d, xi, yi, zi);
            double nb[6];
            int m = 0, c = 6;
            nb[m++] = xv[lin(d, xm1(d, xi), yi, zi)];
            nb[m++] = xv[lin(d, xp1(d, xi), yi, zi)];
            if (d.nz == 1) {
                c = 4;
            } else {
                nb[m++] = xv[lin(d, xi, yi, zm1(d, zi))];
                nb[m++] = xv[lin(d, xi, yi, zp1(d, zi))];
            }
            if (d.channel) {
                if (yi > 0) nb[m++] = xv[lin(d, xi, yi - 1, zi)]; else --c;
                if (yi < d.ny - 1) nb[m++] = xv[lin(d, xi, yi + 1, zi)]; else --c;
            } else {
                nb[m++] = xv[lin(d, xi, ym1(d, yi), zi)];
                nb[m++] = xv[lin(d, xi, yp1(d, yi), zi)];
            }
            const float ri = lap_residual_bfp(b[i], xv[i], nb, m, c, k2);
            r[i] = ri;
            acc += ri * ri;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// One colour of red-black Gauss–Seidel: x_i = (b_i - n^2 S) / (-c n^2).
template <typename T>
__device__ __forceinline__ void rbgs_cell(const Dims& d, T* xv, const T* b, int x, int y, int z, T omega = T(1)) {
    T S, c;
    lap_row(d, xv, x, y, z, S, c);
    const long long i = lin(d, x, y, z);
    const T inv = T(1) / (T(d.n) * T(d.n));
    const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
    T v = (S - b[i] * inv) * rc;
    if (omega != T(1)) v = v + (omega - T(1)) * (v - xv[i]);
    xv[i] = v;
}

// omega != 1: over-relaxed update x + omega (gs - x); omega == 1 is plain
// Gauss-Seidel, bit for bit
template <typename T>
__global__ void k_rbgs(Dims d, int color, T omega, T* __restrict__ xv, const T* __restrict__ b) {
    const int y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    const int x = 2 * (blockIdx.x * BX + threadIdx.x) + ((y + z + color) & 1);
    if (x >= d.nx || y >= d.ny) return;
    rbgs_cell(d, xv, b, x, y, z, omega);
}

// Batched forms: each thread takes ZU cells along z of its (x, y) column and
// computes all of them before storing any, so that ZU cells' loads are in
// flight at once (on GB300 one cell per thread leaves the stencil bound by
// block turnover, near 3 TB/s). Within one colour the red cells read only
// black ones, so the delayed stores change nothing: same values as the
// one-cell kernels.
constexpr int kZU = 8;  // z cells per thread of the batched stencil kernels
constexpr int kZU32 = 4;  // ... of the FP32 red-black colour
// smallest level (x extent) on which a requested over-relaxation applies;
// the coarser levels, the one-block tail among them, stay Gauss-Seidel
constexpr int kOmegaMinNx = 64;

template <typename T, int ZU>
__global__ void k_rbgs_z(Dims d, int color, T omega, T* __restrict__ xv, const T* __restrict__ b) {
    const int y = blockIdx.y * BY + threadIdx.y, t = blockIdx.x * BX + threadIdx.x, z0 = blockIdx.z * ZU;
    if (y >= d.ny) return;
    T val[ZU];
    long long at[ZU];
    const T inv = T(1) / (T(d.n) * T(d.n));
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int z = z0 + u, x = 2 * t + ((y + z + color) & 1);
        at[u] = -1;
        if (x < d.nx) {
            T S, c;
            lap_row(d, xv, x, y, z, S, c);
            const long long i = lin(d, x, y, z);
            const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
            val[u] = (S - b[i] * inv) * rc;
            if (omega != T(1)) val[u] = val[u] + (omega - T(1)) * (val[u] - xv[i]);
            at[u] = i;
        }
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u)
        if (at[u] >= 0) xv[at[u]] = val[u];
}

// Neighbour sum and diagonal factor of lap_row with Ix2 indexing (same terms,
// same order).
template <typename T>
__device__ __forceinline__ void lap_row2(const Dims& d, const Ix2& I, const T* x, int xi, int yi, int zi,
                                         T& S, T& c) {
    if (d.nz == 1) {
        S = x[I.at(I.xm(xi), yi, zi)] + x[I.at(I.xp(xi), yi, zi)];
        c = T(4);
    } else {
        S = (x[I.at(I.xm(xi), yi, zi)] + x[I.at(I.xp(xi), yi, zi)]) + (x[I.at(xi, yi, I.zm(zi))] + x[I.at(xi, yi, I.zp(zi))]);
        c = T(6);
    }
    if (d.channel) {
        if (yi > 0) S += x[I.at(xi, yi - 1, zi)]; else c -= T(1);
        if (yi < d.ny - 1) S += x[I.at(xi, yi + 1, zi)]; else c -= T(1);
    } else {
        S += x[I.at(xi, I.ym(yi), zi)] + x[I.at(xi, I.yp(yi), zi)];
    }
}

template <typename T, int ZU>
__device__ __forceinline__ void rbgs_z2_body(Dims d, int color, T omega, T* __restrict__ xv, const T* __restrict__ b,
                                             int rev) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int y = B.y * BY + threadIdx.y, t = B.x * BX + threadIdx.x, z0 = B.z * ZU;
    if (y >= d.ny || 2 * t >= d.nx) return;
    T val[ZU];
    int at[ZU];
    const T inv = T(1) / (T(d.n) * T(d.n));
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int z = z0 + u, x = 2 * t + ((y + z + color) & 1);
        T S, c;
        lap_row2(d, I, xv, x, y, z, S, c);
        const int i = I.at(x, y, z);
        const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
        val[u] = (S - b[i] * inv) * rc;
        if (omega != T(1)) val[u] = val[u] + (omega - T(1)) * (val[u] - xv[i]);
        at[u] = i;
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) xv[at[u]] = val[u];
}
template <typename T, int ZU>
__global__ void k_rbgs_z2(Dims d, int color, T omega, T* __restrict__ xv, const T* __restrict__ b, int rev) {
    rbgs_z2_body<T, ZU>(d, color, omega, xv, b, rev);
}

// The first colour (red) of a sweep from x = 0 without reading or clearing x
// first: every neighbour is zero, so the neighbour sum lap_row2 forms is the
// zero `zero` (a kernel argument, so that the arithmetic is rbgs_z2_body's,
// not a folded constant) and the update x - 0 the update; the black cell of
// each pair is written as zero. The same bits as a memset of x followed by
// the colour launch.
template <typename T, int ZU, int MINB>
__global__ void __launch_bounds__(BX * BY, MINB) k_rbgs_z2b_init(Dims d, T omega, T* __restrict__ xv,
                                                                const T* __restrict__ b, int rev, T zero) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int y = B.y * BY + threadIdx.y, t = B.x * BX + threadIdx.x, z0 = B.z * ZU;
    if (y >= d.ny || 2 * t >= d.nx) return;
    T val[ZU];
    int at[ZU], other[ZU];
    const T inv = T(1) / (T(d.n) * T(d.n));
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int z = z0 + u, p = (y + z) & 1, x = 2 * t + p;
        T c = d.nz == 1 ? T(4) : T(6);
        if (d.channel) {
            if (!(y > 0)) c -= T(1);
            if (!(y < d.ny - 1)) c -= T(1);
        }
        const int i = I.at(x, y, z);
        const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
        val[u] = (zero - b[i] * inv) * rc;
        if (omega != T(1)) val[u] = val[u] + (omega - T(1)) * (val[u] - zero);
        at[u] = i;
        other[u] = I.at(2 * t + 1 - p, y, z);
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        xv[at[u]] = val[u];
        xv[other[u]] = zero;
    }
}
template <typename T, int ZU, int MINB>
__global__ void __launch_bounds__(BX * BY, MINB) k_rbgs_z2b(Dims d, int color, T omega, T* __restrict__ xv,
                                                           const T* __restrict__ b, int rev) {
    rbgs_z2_body<T, ZU>(d, color, omega, xv, b, rev);
}

// The FP32 colour on float pairs: a thread owns the pairs (2t, 2t+1) of its
// (y, z) column, one cell of each pair being the colour's. Per ZU-cell
// column it loads ZU + 2 pairs of its own column (the z neighbours come from
// the same registers), the pairs of the rows y - 1 and y + 1, and the pairs
// of b: 4.25 eight-byte loads per updated cell, each warp instruction reading
// 256 contiguous bytes, against the scalar kernel's eight stride-2 loads. The
// x neighbour across the pair boundary comes from the adjacent lane by a
// shuffle (the first and last lanes load it). The colour is uniform across a
// warp (its lanes share y and z). The update is rbgs_z2_body's arithmetic in
// the same order, so the same bits; the pair is stored whole, the other
// colour's value unchanged (no thread writes that colour in this launch).
template <int ZU, int MINB>
__global__ void __launch_bounds__(BX * BY, MINB) k_rbgs_pair(Dims d, int color, float omega, float* __restrict__ xv,
                                                            const float* __restrict__ b, int rev) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int t = B.x * BX + threadIdx.x, y = B.y * BY + threadIdx.y, z0 = B.z * ZU;
    const float2* __restrict__ xp = reinterpret_cast<const float2*>(xv);
    const float2* __restrict__ bp = reinterpret_cast<const float2*>(b);
    auto pr = [&](int yy, int zz) { return I.at(2 * t, yy, zz) >> 1; };
    const bool has_lo = !d.channel || y > 0, has_hi = !d.channel || y < d.ny - 1;
    const int ylo = d.channel ? y - 1 : I.ym(y), yhi = d.channel ? y + 1 : I.yp(y);
    float2 col[ZU + 2], ly[ZU], hy[ZU], bb[ZU];
#pragma unroll
    for (int k = 0; k < ZU + 2; ++k) col[k] = xp[pr(y, (z0 - 1 + k) & I.mz)];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        ly[u] = has_lo ? xp[pr(ylo, z0 + u)] : make_float2(0.f, 0.f);
        hy[u] = has_hi ? xp[pr(yhi, z0 + u)] : make_float2(0.f, 0.f);
        bb[u] = bp[pr(y, z0 + u)];
    }
    const float inv = 1.f / (float(d.n) * float(d.n));
    float2 out[ZU];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        const int z = z0 + u, p = (y + z + color) & 1;
        const float2 self = col[u + 1];
        float left, right;
        if (p == 0) {  // the cell 2t: its left neighbour is the previous pair's second value
            float prev = __shfl_up_sync(0xffffffffu, self.y, 1);
            if (threadIdx.x == 0) prev = xv[I.at((2 * t - 1) & I.mx, y, z)];
            left = prev;
            right = self.y;
        } else {  // the cell 2t + 1: its right neighbour is the next pair's first value
            float next = __shfl_down_sync(0xffffffffu, self.x, 1);
            if (threadIdx.x == BX - 1) next = xv[I.at((2 * t + 2) & I.mx, y, z)];
            left = self.x;
            right = next;
        }
        const float zm = p ? col[u].y : col[u].x, zq = p ? col[u + 2].y : col[u + 2].x;
        float S = (left + right) + (zm + zq), c = 6.f;
        const float yl = p ? ly[u].y : ly[u].x, yh = p ? hy[u].y : hy[u].x;
        if (d.channel) {
            if (has_lo) S += yl; else c -= 1.f;
            if (has_hi) S += yh; else c -= 1.f;
        } else {
            S += yl + yh;
        }
        const float rc = (c == 6.f) ? float(1.0 / 6.0) : ((c == 5.f) ? float(1.0 / 5.0) : (c == 4.f ? 0.25f : 1.f / c));
        const float bi = p ? bb[u].y : bb[u].x;
        float v = (S - bi * inv) * rc;
        if (omega != 1.f) v = v + (omega - 1.f) * (v - (p ? self.y : self.x));
        out[u] = p ? make_float2(self.x, v) : make_float2(v, self.y);
    }
    float2* __restrict__ xw = reinterpret_cast<float2*>(xv);
#pragma unroll
    for (int u = 0; u < ZU; ++u) xw[pr(y, z0 + u)] = out[u];
}

template <typename T, int ZU>
__global__ void k_residual_z2(Dims d, T* __restrict__ r, const T* __restrict__ xv, const T* __restrict__ b, int rev) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int x = B.x * BX + threadIdx.x, y = B.y * BY + threadIdx.y, z0 = B.z * ZU;
    if (x >= d.nx || y >= d.ny) return;
    const T off = T(d.n) * T(d.n);
    T val[ZU];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        T S, c;
        lap_row2(d, I, xv, x, y, z0 + u, S, c);
        const int i = I.at(x, y, z0 + u);
        val[u] = b[i] - off * (S - c * xv[i]);
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) r[I.at(x, y, z0 + u)] = val[u];
}

template <typename T, int ZU>
__global__ void k_residual_z(Dims d, T* __restrict__ r, const T* __restrict__ xv, const T* __restrict__ b) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z0 = blockIdx.z * ZU;
    if (x >= d.nx || y >= d.ny) return;
    const T off = T(d.n) * T(d.n);
    T val[ZU];
#pragma unroll
    for (int u = 0; u < ZU; ++u) {
        T S, c;
        lap_row(d, xv, x, y, z0 + u, S, c);
        const long long i = lin(d, x, y, z0 + u);
        val[u] = b[i] - off * (S - c * xv[i]);
    }
#pragma unroll
    for (int u = 0; u < ZU; ++u) r[lin(d, x, y, z0 + u)] = val[u];
}

// ---------------------------------------------------------------------------
// Pipelined red-black sweep: one full sweep (red, then black) per launch, out
// of place (xin -> xout). A block owns FY full-width rows (every x of the row,
// so there is no x halo: x wraps inside shared memory) and a chunk of ZC
// planes, and marches along z. At step k it updates the red cells of plane k
// on the rows tile +- 1, then the black cells of plane k-1 on the tile, then
// writes plane k-1 of the tile. Rows of x (tile +- 2) and of b (tile +- 1)
// arrive in a ring of R = D + 4 plane slots by asynchronous 16-byte copies
// (cp.async) that all threads issue D planes ahead, one commit group per
// plane, so the march does not wait on DRAM. The blocks are persistent and
// take (row strip, z chunk) items in order. Every update is the per-colour
// kernel's arithmetic with the same terms in the same order, so a pipelined
// sweep equals the two per-colour launches cell for cell.
// ---------------------------------------------------------------------------
namespace pipe {
__device__ __forceinline__ unsigned saddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void wait_pending() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
}  // namespace pipe

constexpr int kPipeThreads = 256;

// Gauss-Seidel value of one cell from its six neighbours and b, the
// per-colour kernel's arithmetic (rbgs_cell) in the same order.
template <typename T, bool CH>
__device__ __forceinline__ T gs_value(T xm, T xp, T zm, T zp, T ym, T yp, T bv, T inv, int gy, int ny) {
    T S = (xm + xp) + (zm + zp);
    T c = T(6);
    if (CH) {
        if (gy > 0) S += ym; else c -= T(1);
        if (gy < ny - 1) S += yp; else c -= T(1);
    } else {
        S += ym + yp;
    }
    const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
    return (S - bv * inv) * rc;
}

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    typedef float4 type;
};
template <>
struct Vec4<double> {
    typedef double4 type;
};

// One colour of one plane row segment by quads: the quad of four cells at
// x = 4q .. 4q+3 holds two cells of the colour, at offsets par and par + 2.
template <typename T, bool CH>
__device__ __forceinline__ void gs_quad(T* row, const T* rowm, const T* rowp, const T* zmr, const T* zpr, const T* br,
                                        int q, int nq, int par, T inv, int gy, int ny) {
    typedef typename Vec4<T>::type V;
    V c = reinterpret_cast<V*>(row)[q];
    const V n = reinterpret_cast<const V*>(rowm)[q], s = reinterpret_cast<const V*>(rowp)[q];
    const V a = reinterpret_cast<const V*>(zmr)[q], e = reinterpret_cast<const V*>(zpr)[q];
    const V bb = reinterpret_cast<const V*>(br)[q];
    if (par == 0) {
        const T left = row[4 * (q == 0 ? nq : q) - 1];
        c.x = gs_value<T, CH>(left, c.y, a.x, e.x, n.x, s.x, bb.x, inv, gy, ny);
        c.z = gs_value<T, CH>(c.y, c.w, a.z, e.z, n.z, s.z, bb.z, inv, gy, ny);
    } else {
        const T right = row[q + 1 == nq ? 0 : 4 * (q + 1)];
        c.y = gs_value<T, CH>(c.x, c.z, a.y, e.y, n.y, s.y, bb.y, inv, gy, ny);
        c.w = gs_value<T, CH>(c.z, right, a.w, e.w, n.w, s.w, bb.w, inv, gy, ny);
    }
    reinterpret_cast<V*>(row)[q] = c;
}

// Power-of-two extents only (every level the sweep serves): indices are
// shifts and masks. CH: channel walls in y (Neumann rows, no wrap in y).
template <typename T, int D, bool CH>
__global__ void __launch_bounds__(kPipeThreads, 1) k_rbgs_pipe(Dims d, const T* __restrict__ xin, T* __restrict__ xout,
                                                            const T* __restrict__ b, int FY, int ZC, int lnx, int lny) {
    extern __shared__ __align__(128) unsigned char smem[];
    typedef typename Vec4<T>::type V;
    constexpr int R = D + 4;
    const int nx = d.nx, XR = FY + 4, BR = FY + 2;
    const int xplane = XR * nx, bplane = BR * nx;
    T* xs = (T*)smem;                 // [R][XR][nx]
    T* bs = xs + (size_t)R * xplane;  // [R][BR][nx]
    const int tid = threadIdx.x;
    const int lq = lnx - 2, nq = nx >> 2, qmask = nq - 1;  // quads per row
    const int ymask = d.ny - 1, zmask = d.nz - 1;
    const int lcpr = lnx + (sizeof(T) == 8 ? 3 : 2) - 4;  // log2 of the 16-byte chunks per row
    const int cmask = (1 << lcpr) - 1;
    const T inv = T(1) / (T(d.n) * T(d.n));
    const int nstrip = d.ny / FY, items = nstrip * (d.nz / ZC);
    int s_first = 0;
    auto next_slot = [](int q) { return q + 1 == R ? 0 : q + 1; };
    auto prev_slot = [](int q) { return q == 0 ? R - 1 : q - 1; };
    auto row_ok = [&](int gy) { return !CH || (gy >= 0 && gy < d.ny); };
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int y0 = (item % nstrip) * FY, z0 = (item / nstrip) * ZC, zend = z0 + ZC;
        const int pfirst = z0 - 2, plast = zend + 1;
        auto issue = [&](int p, int q) {
            if (p <= plast) {
                const long long zoff = (long long)(p & zmask) << lny;
                for (int c = tid; c < ((XR + BR) << lcpr); c += kPipeThreads) {
                    const int r = c >> lcpr, o = c & cmask;
                    const bool isx = r < XR;
                    const int gy = isx ? y0 - 2 + r : y0 - 1 + (r - XR);
                    if (!row_ok(gy)) continue;
                    const T* src = (isx ? xin : b) + ((zoff + (gy & ymask)) << lnx);
                    T* dst = isx ? xs + (size_t)q * xplane + (r << lnx) : bs + (size_t)q * bplane + ((r - XR) << lnx);
                    pipe::cp16((char*)dst + 16 * o, (const char*)src + 16 * o);
                }
            }
            pipe::commit();
        };
        int next = pfirst, snext = s_first;
        for (; next <= pfirst + R - 2; ++next, snext = next_slot(snext)) issue(next, snext);
        int skm1 = s_first, sk = next_slot(s_first);
        for (int k = z0 - 1; k <= zend; ++k) {
            const int skp1 = next_slot(sk), skm2 = prev_slot(skm1);
            pipe::wait_pending<D>();
            __syncthreads();
            T* const Xm = xs + (size_t)skm1 * xplane;
            T* const X0 = xs + (size_t)sk * xplane;
            T* const Xp = xs + (size_t)skp1 * xplane;
            {
                // red cells of plane k, rows tile +- 1
                const int gz = k & zmask;
                const T* B0 = bs + (size_t)sk * bplane;
                for (int e = tid; e < ((FY + 2) << lq); e += kPipeThreads) {
                    const int rr = e >> lq, gy = y0 - 1 + rr;
                    if (!row_ok(gy)) continue;
                    const int o = (rr + 1) << lnx;
                    gs_quad<T, CH>(X0 + o, X0 + o - nx, X0 + o + nx, Xm + o, Xp + o, B0 + (rr << lnx), e & qmask, nq,
                                   ((gy & ymask) + gz) & 1, inv, gy, d.ny);
                }
            }
            __syncthreads();
            const int kb = k - 1;
            if (kb >= z0) {
                // black cells of plane k-1 on the tile (z neighbours: k-2 and k)
                const int gz = kb & zmask;
                T* const Ym = xs + (size_t)skm2 * xplane;
                const T* B1 = bs + (size_t)skm1 * bplane;
                for (int e = tid; e < (FY << lq); e += kPipeThreads) {
                    const int rr = e >> lq, gy = y0 + rr;
                    const int o = (rr + 2) << lnx;
                    gs_quad<T, CH>(Xm + o, Xm + o - nx, Xm + o + nx, Ym + o, X0 + o, B1 + ((rr + 1) << lnx), e & qmask,
                                   nq, (gy + gz + 1) & 1, inv, gy, d.ny);
                }
            }
            __syncthreads();
            if (kb >= z0) {
                // plane k-1 of the tile is final
                V* dst = reinterpret_cast<V*>(xout + ((((long long)kb << lny) + y0) << lnx));
                const V* src = reinterpret_cast<const V*>(Xm + 2 * nx);
                for (int e = tid; e < (FY << lq); e += kPipeThreads) dst[e] = src[e];
            }
            // the slot of plane k-2 is free: its last reader, the black update, is behind the barrier
            issue(next, snext);
            ++next;
            snext = next_slot(snext);
            skm1 = sk;
            sk = skp1;
        }
        pipe::wait_pending<0>();
        s_first = (s_first + (next - pfirst)) % R;
        __syncthreads();
    }
}

// Full weighting, src/mg/solver.h:153-181: 64 taps (1,3,3,1)^3/512 around the
// coarse cell; y clamps at the channel walls, wraps in periodic mode.
template <typename T>
__device__ __forceinline__ void restrict_cell(const Dims& d, T* coarse, const T* fine, int xc, int yc, int zc) {
    const int cx = d.nx / 2, cy = d.ny / 2;
    if (d.nz == 1) {
        // 2D (periodic): (1,3,3,1)^2 / 64 over 16 taps
        const T wgt[4] = {T(1), T(3), T(3), T(1)};
        T acc = T(0);
#pragma unroll
        for (int ky = 0; ky < 4; ++ky)
#pragma unroll
            for (int kx = 0; kx < 4; ++kx)
                acc += (wgt[kx] * wgt[ky] / T(64)) *
                       fine[lin(d, wrapi(2 * xc + 1 + kx - 2, d.nx), wrapi(2 * yc + 1 + ky - 2, d.ny), 0)];
        coarse[xc + (long long)cx * yc] = acc;
        return;
    }
    const int xcf = 2 * xc + 1, ycf = 2 * yc + 1, zcf = 2 * zc + 1;
    int xs[4], ys[4], zs[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int dd = k - 2;
        xs[k] = wrapi(xcf + dd, d.nx);
        zs[k] = wrapi(zcf + dd, d.nz);
        if (d.channel) {
            int yy = ycf + (dd > -ycf ? dd : -ycf);
            ys[k] = yy < d.ny - 1 ? yy : d.ny - 1;
        } else {
            ys[k] = wrapi(ycf + dd, d.ny);
        }
    }
    const T wgt[4] = {T(1), T(3), T(3), T(1)};
    T acc = T(0);
#pragma unroll
    for (int kz = 0; kz < 4; ++kz)
#pragma unroll
        for (int ky = 0; ky < 4; ++ky)
#pragma unroll
            for (int kx = 0; kx < 4; ++kx)
                acc += (wgt[kx] * wgt[ky] * wgt[kz] / T(512)) * fine[lin(d, xs[kx], ys[ky], zs[kz])];
    coarse[xc + (long long)cx * (yc + (long long)cy * zc)] = acc;
}

// zero (optional): the coarse iterate, set to zero at every coarse cell
template <typename T>
__global__ void k_restrict(Dims d, T* __restrict__ coarse, const T* __restrict__ fine, T* __restrict__ zero) {
    const int xc = blockIdx.x * BX + threadIdx.x, yc = blockIdx.y * BY + threadIdx.y, zc = blockIdx.z;
    if (xc >= d.nx / 2 || yc >= d.ny / 2) return;
    restrict_cell(d, coarse, fine, xc, yc, zc);
    if (zero) {
        const long long cx = d.nx / 2, cy = d.ny / 2;
        zero[d.nz == 1 ? xc + cx * yc : xc + cx * (yc + cy * zc)] = T(0);
    }
}

// Trilinear prolongation (27,9,3,1)/64, src/mg/solver.h:71-151. One thread per
// coarse cell writes the eight fine cells between it and its +1 neighbours;
// in channel mode the wall rows take the bilinear (9,3,1)/16 weights.
template <typename T, bool ADD>
__device__ __forceinline__ void prolong_cell(const Dims& d, T* fine, const T* coarse, int xc, int yc, int zc) {
    const int cx = d.nx / 2, cy = d.ny / 2, cz = d.nz / 2;
    auto C = [&](int a, int b, int c) { return coarse[a + (long long)cx * (b + (long long)cy * c)]; };
    auto put = [&](int a, int b, int c, T val) {
        const long long i = lin(d, a, b, c);
        if (ADD) fine[i] = fine[i] + val; else fine[i] = val;
    };
    if (d.nz == 1) {
        // 2D (periodic): bilinear (9,3,3,1)/16 onto the four fine cells
        auto C2 = [&](int a, int b) { return coarse[a + (long long)cx * b]; };
        const int xn = (xc + 1) % cx, yn = (yc + 1) % cy;
        const int xcf = 2 * xc + 1, ycf = 2 * yc + 1, xnf = (xcf + 1) % d.nx, ynf = (ycf + 1) % d.ny;
        const T bl = C2(xc, yc), br = C2(xn, yc), ul = C2(xc, yn), ur = C2(xn, yn);
        const T a = T(9) / T(16), b = T(3) / T(16), e = T(1) / T(16);
        put(xcf, ycf, 0, a * bl + b * (br + ul) + e * ur);
        put(xnf, ycf, 0, a * br + b * (bl + ur) + e * ul);
        put(xcf, ynf, 0, a * ul + b * (ur + bl) + e * br);
        put(xnf, ynf, 0, a * ur + b * (ul + br) + e * bl);
        return;
    }
    const int xn = (xc + 1) % cx, zn = (zc + 1) % cz;
    const int xcf = 2 * xc + 1, zcf = 2 * zc + 1;
    const int xnf = (xcf + 1) % d.nx, znf = (zcf + 1) % d.nz;
    const bool interior = d.channel ? (yc < cy - 1) : true;
    if (interior) {
        const int yn = d.channel ? yc + 1 : (yc + 1) % cy;
        const int ycf = 2 * yc + 1, ynf = d.channel ? ycf + 1 : (ycf + 1) % d.ny;
        const T blb = C(xc, yc, zc), brb = C(xn, yc, zc), ulb = C(xc, yn, zc), urb = C(xn, yn, zc);
        const T blf = C(xc, yc, zn), brf = C(xn, yc, zn), ulf = C(xc, yn, zn), urf = C(xn, yn, zn);
        const T a = T(27) / T(64), b = T(9) / T(64), c = T(3) / T(64), e = T(1) / T(64);
        put(xcf, ycf, zcf, a * blb + b * (brb + ulb + blf) + c * (urb + ulf + brf) + e * urf);
        put(xnf, ycf, zcf, a * brb + b * (urb + blb + brf) + c * (ulb + blf + urf) + e * ulf);
        put(xcf, ynf, zcf, a * ulb + b * (urb + blb + ulf) + c * (brb + blf + urf) + e * brf);
        put(xnf, ynf, zcf, a * urb + b * (brb + ulb + urf) + c * (blb + ulf + brf) + e * blf);
        put(xcf, ycf, znf, a * blf + b * (brf + ulf + blb) + c * (urf + ulb + brb) + e * urb);
        put(xnf, ycf, znf, a * brf + b * (urf + blf + brb) + c * (ulf + blb + urb) + e * ulb);
        put(xcf, ynf, znf, a * ulf + b * (urf + blf + ulb) + c * (brf + blb + urb) + e * brb);
        put(xnf, ynf, znf, a * urf + b * (brf + ulf + urb) + c * (blf + ulb + brb) + e * blb);
    }
    if (d.channel && (yc == 0 || yc == cy - 1)) {
        const T a = T(9) / T(16), b = T(3) / T(16), e = T(1) / T(16);
        // a thread with cy == 1 owns both wall rows
        for (int side = 0; side < 2; ++side) {
            if (side == 0 && yc != 0) continue;
            if (side == 1 && yc != cy - 1) continue;
            const int ycs = side == 0 ? 0 : cy - 1, yf = side == 0 ? 0 : d.ny - 1;
            const T bl = C(xc, ycs, zc), br = C(xn, ycs, zc), fl = C(xc, ycs, zn), fr = C(xn, ycs, zn);
            put(xcf, yf, zcf, a * bl + b * (br + fl) + e * fr);
            put(xnf, yf, zcf, a * br + b * (bl + fr) + e * fl);
            put(xcf, yf, znf, a * fl + b * (fr + bl) + e * br);
            put(xnf, yf, znf, a * fr + b * (fl + br) + e * bl);
        }
    }
}

// restrict_cell / prolong_cell for 3D power-of-two levels with Ix2 indexing
// (same taps, same weights, same summation order)
template <typename T>
__device__ __forceinline__ void restrict_cell2(const Dims& d, const Ix2& I, T* coarse, const T* fine, int xc, int yc,
                                               int zc) {
    const int xcf = 2 * xc + 1, ycf = 2 * yc + 1, zcf = 2 * zc + 1;
    int xs[4], yo[4], zo[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int dd = k - 2;
        xs[k] = (xcf + dd) & I.mx;
        zo[k] = ((zcf + dd) & I.mz) << I.lxy;
        if (d.channel) {
            int yy = ycf + (dd > -ycf ? dd : -ycf);
            yo[k] = (yy < d.ny - 1 ? yy : d.ny - 1) << I.lx;
        } else {
            yo[k] = ((ycf + dd) & I.my) << I.lx;
        }
    }
    const T wgt[4] = {T(1), T(3), T(3), T(1)};
    T acc = T(0);
#pragma unroll
    for (int kz = 0; kz < 4; ++kz)
#pragma unroll
        for (int ky = 0; ky < 4; ++ky)
#pragma unroll
            for (int kx = 0; kx < 4; ++kx)
                acc += (wgt[kx] * wgt[ky] * wgt[kz] / T(512)) * fine[xs[kx] | yo[ky] | zo[kz]];
    coarse[xc | (yc << (I.lx - 1)) | (zc << (I.lxy - 2))] = acc;
}

template <typename T>
__global__ void k_restrict2(Dims d, T* __restrict__ coarse, const T* __restrict__ fine, int rev,
                            T* __restrict__ zero) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int xc = B.x * BX + threadIdx.x, yc = B.y * BY + threadIdx.y, zc = B.z;
    if (xc >= d.nx / 2 || yc >= d.ny / 2) return;
    restrict_cell2(d, I, coarse, fine, xc, yc, zc);
    if (zero) zero[xc | (yc << (I.lx - 1)) | (zc << (I.lxy - 2))] = T(0);
}

template <typename T, bool ADD>
__device__ __forceinline__ void prolong_cell2(const Dims& d, const Ix2& I, T* fine, const T* coarse, int xc, int yc,
                                              int zc) {
    const int cx = d.nx / 2, cy = d.ny / 2, cz = d.nz / 2, lcx = I.lx - 1, lcxy = I.lxy - 2;
    auto C = [&](int a, int b, int c) { return coarse[a | (b << lcx) | (c << lcxy)]; };
    auto put = [&](int a, int b, int c, T val) {
        const int i = I.at(a, b, c);
        if (ADD) fine[i] = fine[i] + val; else fine[i] = val;
    };
    const int xn = (xc + 1) & (cx - 1), zn = (zc + 1) & (cz - 1);
    const int xcf = 2 * xc + 1, zcf = 2 * zc + 1;
    const int xnf = (xcf + 1) & I.mx, znf = (zcf + 1) & I.mz;
    const bool interior = d.channel ? (yc < cy - 1) : true;
    if (interior) {
        const int yn = d.channel ? yc + 1 : (yc + 1) & (cy - 1);
        const int ycf = 2 * yc + 1, ynf = d.channel ? ycf + 1 : (ycf + 1) & I.my;
        const T blb = C(xc, yc, zc), brb = C(xn, yc, zc), ulb = C(xc, yn, zc), urb = C(xn, yn, zc);
        const T blf = C(xc, yc, zn), brf = C(xn, yc, zn), ulf = C(xc, yn, zn), urf = C(xn, yn, zn);
        const T a = T(27) / T(64), b = T(9) / T(64), c = T(3) / T(64), e = T(1) / T(64);
        put(xcf, ycf, zcf, a * blb + b * (brb + ulb + blf) + c * (urb + ulf + brf) + e * urf);
        put(xnf, ycf, zcf, a * brb + b * (urb + blb + brf) + c * (ulb + blf + urf) + e * ulf);
        put(xcf, ynf, zcf, a * ulb + b * (urb + blb + ulf) + c * (brb + blf + urf) + e * brf);
        put(xnf, ynf, zcf, a * urb + b * (brb + ulb + urf) + c * (blb + ulf + brf) + e * blf);
        put(xcf, ycf, znf, a * blf + b * (brf + ulf + blb) + c * (urf + ulb + brb) + e * urb);
        put(xnf, ycf, znf, a * brf + b * (urf + blf + brb) + c * (ulf + blb + urb) + e * ulb);
        put(xcf, ynf, znf, a * ulf + b * (urf + blf + ulb) + c * (brf + blb + urb) + e * brb);
        put(xnf, ynf, znf, a * urf + b * (brf + ulf + urb) + c * (blf + ulb + brb) + e * blb);
    }
    if (d.channel && (yc == 0 || yc == cy - 1)) {
        const T a = T(9) / T(16), b = T(3) / T(16), e = T(1) / T(16);
        for (int side = 0; side < 2; ++side) {
            if (side == 0 && yc != 0) continue;
            if (side == 1 && yc != cy - 1) continue;
            const int ycs = side == 0 ? 0 : cy - 1, yf = side == 0 ? 0 : d.ny - 1;
            const T bl = C(xc, ycs, zc), br = C(xn, ycs, zc), fl = C(xc, ycs, zn), fr = C(xn, ycs, zn);
            put(xcf, yf, zcf, a * bl + b * (br + fl) + e * fr);
            put(xnf, yf, zcf, a * br + b * (bl + fr) + e * fl);
            put(xcf, yf, znf, a * fl + b * (fr + bl) + e * br);
            put(xnf, yf, znf, a * fr + b * (fl + br) + e * bl);
        }
    }
}

// Fine-level residual fused with the full-weighting restriction and the
// zeroing of the coarse iterate. A block takes RR_T x RR_T coarse columns
// and RR_CZ coarse planes; r = b - L x of its fine tile (2 RR_T + 2 cells a
// side: the taps reach one fine cell beyond the tile's own) is formed in
// shared memory, one fine plane at a time, in a ring of the four planes the
// current coarse plane reads, and every coarse cell sums its 64 taps from the
// ring. The residual is k_residual_z2's expression and the taps are
// restrict_cell2's in its order, so the coarse right-hand side equals the two
// kernels' bit for bit, and the fine residual is never written to memory.
constexpr int RR_T = 16, RR_F = 2 * RR_T + 2, RR_THREADS = RR_T * RR_T;
// ring plane layout: row stride RR_RS, even columns first and odd columns
// from RR_ODD, so that the 16 coarse cells of a half warp read 16
// consecutive words and the two halves (two fine rows apart) the other 16
// banks: no shared-memory bank conflicts in the tap loop
constexpr int RR_RS = 40, RR_ODD = 20;
__device__ __forceinline__ int rr_at(int jy, int jx) { return jy * RR_RS + (jx & 1) * RR_ODD + (jx >> 1); }

template <typename T, int RR_CZ>
__global__ void __launch_bounds__(RR_THREADS) k_resid_restrict2(Dims d, T* __restrict__ cb, T* __restrict__ cx,
                                                               const T* __restrict__ xv, const T* __restrict__ b,
                                                               int rev) {
    __shared__ T ring[4][RR_F * RR_RS];
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int xc0 = B.x * RR_T, yc0 = B.y * RR_T, zc0 = B.z * RR_CZ;
    const int xf0 = 2 * xc0 - 1, yf0 = 2 * yc0 - 1;  // fine cell of tile column / row 0 (unwrapped)
    const T off = T(d.n) * T(d.n);
    const int tid = threadIdx.x;
    // residual of fine plane zf (unwrapped) into its ring slot; channel rows
    // beyond the walls are never tapped (the taps clamp) and stay unset
    auto fill = [&](int zf) {
        T* dst = ring[zf & 3];
        const int z = zf & I.mz;
        for (int e = tid; e < RR_F * RR_F; e += RR_THREADS) {
            const int jy = e / RR_F, jx = e - jy * RR_F;
            int y = yf0 + jy;
            if (d.channel) {
                if (y < 0 || y >= d.ny) continue;
            } else {
                y &= I.my;
            }
            const int x = (xf0 + jx) & I.mx;
            T S, c;
            lap_row2(d, I, xv, x, y, z, S, c);
            const int i = I.at(x, y, z);
            dst[rr_at(jy, jx)] = b[i] - off * (S - c * xv[i]);
        }
    };
    const int cxl = tid % RR_T, cyl = tid / RR_T;
    const int xc = xc0 + cxl, yc = yc0 + cyl;
    int col[4], row[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int dd = k - 2;
        col[k] = (k & 1) * RR_ODD + cxl + (k >> 1);  // tile column 2 cxl + k: fine x = 2 xc + 1 + dd
        int yy;
        if (d.channel) {
            const int ycf = 2 * yc + 1;
            yy = ycf + (dd > -ycf ? dd : -ycf);
            yy = yy < d.ny - 1 ? yy : d.ny - 1;
        } else {
            yy = 2 * yc + 1 + dd;  // unwrapped: the ring holds the wrapped values in order
        }
        row[k] = yy - yf0;
    }
    const T wgt[4] = {T(1), T(3), T(3), T(1)};
    fill(2 * zc0 - 1);
    fill(2 * zc0);
    for (int zc = zc0; zc < zc0 + RR_CZ; ++zc) {
        fill(2 * zc + 1);
        fill(2 * zc + 2);
        __syncthreads();
        T acc = T(0);
#pragma unroll
        for (int kz = 0; kz < 4; ++kz) {
            const T* pl = ring[(2 * zc - 1 + kz) & 3];
#pragma unroll
            for (int ky = 0; ky < 4; ++ky)
#pragma unroll
                for (int kx = 0; kx < 4; ++kx)
                    acc += (wgt[kx] * wgt[ky] * wgt[kz] / T(512)) * pl[row[ky] * RR_RS + col[kx]];
        }
        const int o = xc | (yc << (I.lx - 1)) | (zc << (I.lxy - 2));
        cb[o] = acc;
        cx[o] = T(0);
        __syncthreads();  // the next fills overwrite the two oldest planes
    }
}

template <typename T, bool ADD>
__global__ void k_prolong2(Dims d, T* __restrict__ fine, const T* __restrict__ coarse, int rev) {
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int xc = B.x * BX + threadIdx.x, yc = B.y * BY + threadIdx.y, zc = B.z;
    if (xc >= d.nx / 2 || yc >= d.ny / 2) return;
    prolong_cell2<T, ADD>(d, I, fine, coarse, xc, yc, zc);
}

template <typename T, bool ADD>
__global__ void k_prolong(Dims d, T* __restrict__ fine, const T* __restrict__ coarse) {
    const int xc = blockIdx.x * BX + threadIdx.x, yc = blockIdx.y * BY + threadIdx.y, zc = blockIdx.z;
    if (xc >= d.nx / 2 || yc >= d.ny / 2) return;
    prolong_cell<T, ADD>(d, fine, coarse, xc, yc, zc);
}

// Column-marching transfers for 3D power-of-two levels whose coarse x extent
// is a multiple of 32 and coarse y extent a multiple of kTrBY. A warp holds 32
// consecutive coarse x of one coarse row, so its fine accesses are the 64
// consecutive cells 2 xc .. 2 xc + 63 of a fine row, read or written as one
// pair per lane (256 contiguous bytes for FP32); the cells one beyond a lane's
// pair come from the adjacent lane by a shuffle (the first and last lanes load
// them). A thread then walks CZ coarse planes along z. The one-cell kernels
// (restrict_cell2, prolong_cell2) read and write with a stride of two cells,
// 64 single loads per coarse cell in the restriction, and their prolongation
// stores wait on the loads of the next cell (same array): on 256^3 both ran at
// a third of the copy bandwidth.
constexpr int kTrBY = 8;
template <typename T>
struct Pair;
template <>
struct Pair<float> {
    using type = float2;
};
template <>
struct Pair<double> {
    using type = double2;
};

// Full weighting with restrict_cell2's taps, weights and summation order: the
// coarse cell's single accumulator takes its 64 terms plane by plane (kz), row
// by row (ky), cell by cell (kx). Fine planes 2 zc + 1 and 2 zc + 2 are the
// last two planes (kz = 2, 3) of coarse plane zc and the first two (kz = 0, 1)
// of zc + 1, so each fine plane is read once and feeds two accumulators, the
// second of which starts from zero with that plane's terms: the same
// additions in the same order as the one-cell kernel, the same bits.
//
// A lane reads 16 bytes of each fine tap row (CE = 4 FP32 or 2 FP64 cells)
// and takes the cells on either side from its neighbours, so it serves CE / 2
// coarse cells: a warp covers 16 CE coarse x. The block's fine tile of a plane
// (rows 2 yc0 - 1 .. 2 yc0 + 16, clamped at channel walls, wrapped otherwise;
// 32 CE cells from 2 xc0 and one 16-byte chunk on either side, wrapped in x)
// arrives in shared memory by 16-byte asynchronous copies issued
// kTrStages - 1 planes ahead, one commit group per plane, so that the march
// along z keeps two planes of DRAM reads in flight with one barrier per plane.
constexpr int kTrStages = 3;
constexpr int kTrRows = 2 * kTrBY + 2;
template <typename T>
struct TrTile {
    static constexpr int CE = 16 / (int)sizeof(T);       // cells per 16-byte chunk (per lane)
    static constexpr int CX = 16 * CE;                    // coarse x per block
    static constexpr int W = 34 * CE;                     // row: left chunk, 32 lane chunks, right chunk
    static constexpr int CHUNKS = kTrRows * 34;           // 16-byte chunks per plane
    static constexpr int PER_THREAD = (CHUNKS + 32 * kTrBY - 1) / (32 * kTrBY);
};
template <typename T>
struct Quad;
template <>
struct Quad<float> {
    using type = float4;
};
template <>
struct Quad<double> {
    using type = double2;
};
template <typename T>
__device__ __forceinline__ void quad_get(const T* p, T (&v)[16 / sizeof(T)]) {
    const typename Quad<T>::type q = *reinterpret_cast<const typename Quad<T>::type*>(p);
    if constexpr (sizeof(T) == 4) {
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
        v[0] = q.x; v[1] = q.y;
    }
}

template <typename T, int CZ>
__global__ void __launch_bounds__(32 * kTrBY) k_restrict_cols(Dims d, T* __restrict__ coarse,
                                                              const T* __restrict__ fine, int rev,
                                                              T* __restrict__ zero) {
    using TT = TrTile<T>;
    constexpr int CE = TT::CE, M = CE / 2;  // M coarse cells per lane
    constexpr int NP = 2 * CZ + 2;          // fine planes of the block
    __shared__ __align__(16) T st[kTrStages][kTrRows * TT::W];
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
    const int xc0 = B.x * TT::CX, yc0 = B.y * kTrBY, zc0 = B.z * CZ;
    // this thread's chunks of every plane: source offset within the plane
    // (-1: none) and destination offset within the stage
    int src[TT::PER_THREAD], dst[TT::PER_THREAD];
#pragma unroll
    for (int u = 0; u < TT::PER_THREAD; ++u) {
        const int c = tid + u * 32 * kTrBY;
        src[u] = -1;
        dst[u] = 0;
        if (c < TT::CHUNKS) {
            const int j = c / 34, k = c - j * 34;
            int y = 2 * yc0 - 1 + j;
            if (d.channel) y = y < 0 ? 0 : (y > d.ny - 1 ? d.ny - 1 : y);
            else y &= I.my;
            src[u] = ((2 * xc0 - CE + k * CE) & I.mx) | (y << I.lx);
            dst[u] = j * TT::W + k * CE;
        }
    }
    // copies of fine plane 2 zc0 - 1 + i; a commit group per plane, empty
    // past the block's last plane, so that the group count is the plane count
    auto issue = [&](int i) {
        if (i < NP) {
            T* stage = st[i % kTrStages];
            const T* pl = fine + (((2 * zc0 - 1 + i) & I.mz) << I.lxy);
#pragma unroll
            for (int u = 0; u < TT::PER_THREAD; ++u)
                if (src[u] >= 0) pipe::cp16(stage + dst[u], pl + src[u]);
        }
        pipe::commit();
    };
    auto acquire = [&](int i) -> const T* {
        pipe::wait_pending<kTrStages - 2>();
        __syncthreads();           // plane i is in; plane i - 1 is read by every thread
        issue(i + kTrStages - 1);  // into plane i - 1's stage
        return st[i % kTrStages];
    };
    // the taps of a staged plane: e[ky][1 + q] = fine x = 2 xc0 + CE lane + q,
    // q = -1 .. CE (rows 2 ty + ky of the tile)
    auto taps = [&](const T* pl, T (&e)[4][CE + 2]) {
#pragma unroll
        for (int ky = 0; ky < 4; ++ky) {
            const T* row = pl + (2 * ty + ky) * TT::W + CE;  // fine x = 2 xc0
            T v[CE];
            quad_get(row + CE * lane, v);
            T l = __shfl_up_sync(0xffffffffu, v[CE - 1], 1), r = __shfl_down_sync(0xffffffffu, v[0], 1);
            if (lane == 0) l = row[-1];
            if (lane == 31) r = row[32 * CE];
            e[ky][0] = l;
#pragma unroll
            for (int q = 0; q < CE; ++q) e[ky][1 + q] = v[q];
            e[ky][CE + 1] = r;
        }
    };
    const T wgt[4] = {T(1), T(3), T(3), T(1)};
    // coarse cell m of the lane: taps fine x = 2 xc - 1 .. 2 xc + 2 = e[ky][2m .. 2m + 3]
    auto add = [&](T (&acc)[M], const T (&e)[4][CE + 2], int kz) {
#pragma unroll
        for (int m = 0; m < M; ++m)
#pragma unroll
            for (int ky = 0; ky < 4; ++ky)
#pragma unroll
                for (int kx = 0; kx < 4; ++kx) acc[m] += (wgt[kx] * wgt[ky] * wgt[kz] / T(512)) * e[ky][2 * m + kx];
    };
#pragma unroll
    for (int i = 0; i < kTrStages - 1; ++i) issue(i);
    T acc[M], next[M], e[4][CE + 2];
#pragma unroll
    for (int m = 0; m < M; ++m) acc[m] = T(0);
    taps(acquire(0), e);
    add(acc, e, 0);
    taps(acquire(1), e);
    add(acc, e, 1);
    const int co = (xc0 + M * lane) | ((yc0 + ty) << (I.lx - 1));
    for (int k = 0; k < CZ; ++k) {
#pragma unroll
        for (int m = 0; m < M; ++m) next[m] = T(0);
        taps(acquire(2 * k + 2), e);
        add(acc, e, 2);
        add(next, e, 0);
        taps(acquire(2 * k + 3), e);
        add(acc, e, 3);
        add(next, e, 1);
        const int o = co | ((zc0 + k) << (I.lxy - 2));
        if constexpr (M == 2) {
            *reinterpret_cast<float2*>(coarse + o) = make_float2(acc[0], acc[1]);
            if (zero) *reinterpret_cast<float2*>(zero + o) = make_float2(0.f, 0.f);
        } else {
            coarse[o] = acc[0];
            if (zero) zero[o] = T(0);
        }
#pragma unroll
        for (int m = 0; m < M; ++m) acc[m] = next[m];
    }
    pipe::wait_pending<0>();
}

// FP32 fine-level residual fused with the column restriction: the block of
// k_restrict_cols (64 coarse x, kTrBY coarse y, CZ coarse planes) forms the
// residual r = b - L x of each fine plane of its tile in shared memory and
// restricts from there, so the fine residual never goes to memory. x planes
// (rows 2 yc0 - 2 .. 2 yc0 + 17, 36 16-byte chunks a row from x = 2 xc0 - 8)
// and b planes (rows 2 yc0 - 1 .. 2 yc0 + 16, 34 chunks from 2 xc0 - 4)
// arrive by asynchronous copies issued two planes ahead into rings of kRrX
// and kRrB slots; per fine plane there are two barriers (the plane's inputs
// are in and the previous taps are done / the residual plane is written).
// The residual plane holds 34 chunks a row (x = 2 xc0 - 4 .. 2 xc0 + 131, the
// layout k_restrict_cols stages): each thread forms whole chunks, four cells
// from 16-byte words and the cells on either side by single loads. Every
// residual is k_residual_z2's expression in its order and the taps are
// k_restrict_cols' (restrict_cell2's order), so the coarse right-hand side
// equals the two kernels' bit for bit. In channel mode the rows beyond the
// walls take the residual of the wall row, as the restriction's clamped taps
// read it.
constexpr int kRrX = 4, kRrB = 4, kRrXRows = 2 * kTrBY + 4;
constexpr int kRrXW = 144, kRrW = 136;  // floats a staged x row (36 chunks) / b and residual row (34)
constexpr int kRrTasks = kTrRows * 34;  // residual chunks a plane
constexpr int kRrPT = (kRrTasks + 32 * kTrBY - 1) / (32 * kTrBY);
constexpr size_t kRrSmem = sizeof(float) * ((size_t)kRrX * kRrXRows * kRrXW + (size_t)kRrB * kTrRows * kRrW +
                                            (size_t)kTrRows * kRrW);

template <int CZ, bool CH>
__global__ void __launch_bounds__(32 * kTrBY, 2) k_resid_restrict_cols(Dims d, float* __restrict__ cb,
                                                                    float* __restrict__ cxz,
                                                                    const float* __restrict__ xv,
                                                                    const float* __restrict__ bv, int rev) {
    constexpr int NP = 2 * CZ + 2;  // fine planes restricted (residuals formed)
    constexpr int NI = NP + 2;      // staged items: x planes 2 zc0 - 2 .. 2 zc0 + 2 CZ + 1
    constexpr int XCH = (kRrXRows * 36 + 32 * kTrBY - 1) / (32 * kTrBY);
    constexpr int BCH = (kTrRows * 34 + 32 * kTrBY - 1) / (32 * kTrBY);
    extern __shared__ __align__(16) float rr_smem[];
    float* xs = rr_smem;                          // [kRrX][kRrXRows][kRrXW]
    float* bs = xs + kRrX * kRrXRows * kRrXW;     // [kRrB][kTrRows][kRrW]
    float* rs = bs + kRrB * kTrRows * kRrW;       // [kTrRows][kRrW]
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
    const int xc0 = B.x * 64, yc0 = B.y * kTrBY, zc0 = B.z * CZ;
    auto yrow = [&](int y) {  // a row in range: clamped at channel walls, wrapped otherwise
        if (CH) return y < 0 ? 0 : (y > d.ny - 1 ? d.ny - 1 : y);
        return y & I.my;
    };
    // this thread's chunks of every x / b plane: source offset within the
    // plane (-1: none), destination offset within the slot
    int xsrc[XCH], xdst[XCH], bsrc[BCH], bdst[BCH];
#pragma unroll
    for (int u = 0; u < XCH; ++u) {
        const int c = tid + u * 32 * kTrBY;
        xsrc[u] = -1;
        xdst[u] = 0;
        if (c < kRrXRows * 36) {
            const int j = c / 36, k = c - j * 36;
            xsrc[u] = ((2 * xc0 - 8 + 4 * k) & I.mx) | (yrow(2 * yc0 - 2 + j) << I.lx);
            xdst[u] = j * kRrXW + 4 * k;
        }
    }
#pragma unroll
    for (int u = 0; u < BCH; ++u) {
        const int c = tid + u * 32 * kTrBY;
        bsrc[u] = -1;
        bdst[u] = 0;
        if (c < kTrRows * 34) {
            const int j = c / 34, k = c - j * 34;
            bsrc[u] = ((2 * xc0 - 4 + 4 * k) & I.mx) | (yrow(2 * yc0 - 1 + j) << I.lx);
            bdst[u] = j * kRrW + 4 * k;
        }
    }
    // this thread's residual chunks: residual row jr, chunk k (cells
    // x = 2 xc0 - 4 + 4 k ..); the x-tile row of the residual's row (channel:
    // the wall row for the rows beyond it) and its wall flags
    int tr[kRrPT], tx[kRrPT], tb[kRrPT];
    bool tym[kRrPT], typ[kRrPT];
#pragma unroll
    for (int u = 0; u < kRrPT; ++u) {
        const int t = tid + u * 32 * kTrBY;
        tr[u] = -1;
        tx[u] = 0;
        tb[u] = 0;
        tym[u] = typ[u] = true;
        if (t < kRrTasks) {
            const int jr = t / 34, k = t - jr * 34;
            const int y = 2 * yc0 - 1 + jr;
            const int ye = CH ? (y < 0 ? 0 : (y > d.ny - 1 ? d.ny - 1 : y)) : y;
            const int jx = ye - (2 * yc0 - 2);
            tr[u] = jr * kRrW + 4 * k;
            tb[u] = jr * kRrW + 4 * k;
            tx[u] = jx * kRrXW + 4 * k + 4;
            tym[u] = !CH || ye > 0;
            typ[u] = !CH || ye < d.ny - 1;
        }
    }
    // item k: x plane 2 zc0 - 2 + k, and b of the same plane for 1 <= k <= NP;
    // one commit group per item, empty past the last
    auto issue = [&](int k) {
        if (k < NI) {
            const int zo = ((2 * zc0 - 2 + k) & I.mz) << I.lxy;
            float* xd = xs + (k % kRrX) * kRrXRows * kRrXW;
            const float* xsp = xv + zo;
#pragma unroll
            for (int u = 0; u < XCH; ++u)
                if (xsrc[u] >= 0) pipe::cp16(xd + xdst[u], xsp + xsrc[u]);
            if (k >= 1 && k <= NP) {
                float* bd = bs + (k % kRrB) * kTrRows * kRrW;
                const float* bsp = bv + zo;
#pragma unroll
                for (int u = 0; u < BCH; ++u)
                    if (bsrc[u] >= 0) pipe::cp16(bd + bdst[u], bsp + bsrc[u]);
            }
        }
        pipe::commit();
    };
    const float off = float(d.n) * float(d.n);
    auto cell = [&](float x0, float xl, float xr, float zm, float zp, float ym, float yp, float b, bool hm, bool hp) {
        float S = (xl + xr) + (zm + zp);
        float c = 6.f;
        if (CH) {
            if (hm) S += ym; else c -= 1.f;
            if (hp) S += yp; else c -= 1.f;
        } else {
            S += ym + yp;
        }
        return b - off * (S - c * x0);
    };
    // residual chunks of fine plane i (fine z = 2 zc0 - 1 + i) into rs
    auto resid = [&](int i) {
        const float* xc = xs + ((i + 1) % kRrX) * kRrXRows * kRrXW;
        const float* xm = xs + (i % kRrX) * kRrXRows * kRrXW;        // z - 1
        const float* xp = xs + ((i + 2) % kRrX) * kRrXRows * kRrXW;  // z + 1
        const float* bp = bs + ((i + 1) % kRrB) * kTrRows * kRrW;
#pragma unroll
        for (int u = 0; u < kRrPT; ++u) {
            if (tr[u] < 0) break;
            const float* c0 = xc + tx[u];
            const float4 v = *reinterpret_cast<const float4*>(c0);
            const float4 vym = *reinterpret_cast<const float4*>(c0 - kRrXW);
            const float4 vyp = *reinterpret_cast<const float4*>(c0 + kRrXW);
            const float4 vzm = *reinterpret_cast<const float4*>(xm + tx[u]);
            const float4 vzp = *reinterpret_cast<const float4*>(xp + tx[u]);
            const float4 vb = *reinterpret_cast<const float4*>(bp + tb[u]);
            const float l = c0[-1], r = c0[4];
            const bool hm = tym[u], hp = typ[u];
            float4 o;
            o.x = cell(v.x, l, v.y, vzm.x, vzp.x, vym.x, vyp.x, vb.x, hm, hp);
            o.y = cell(v.y, v.x, v.z, vzm.y, vzp.y, vym.y, vyp.y, vb.y, hm, hp);
            o.z = cell(v.z, v.y, v.w, vzm.z, vzp.z, vym.z, vyp.z, vb.z, hm, hp);
            o.w = cell(v.w, v.z, r, vzm.w, vzp.w, vym.w, vyp.w, vb.w, hm, hp);
            *reinterpret_cast<float4*>(rs + tr[u]) = o;
        }
    };
    const float wgt[4] = {1.f, 3.f, 3.f, 1.f};
    // the restriction taps of the residual plane for this thread: e[ky][1 + q]
    // = fine x = 2 xc0 + 4 lane + q, q = -1 .. 4 (k_restrict_cols' taps)
    auto taps = [&](float (&e)[4][6]) {
#pragma unroll
        for (int ky = 0; ky < 4; ++ky) {
            const float* row = rs + (2 * ty + ky) * kRrW + 4;  // fine x = 2 xc0
            const float4 q = *reinterpret_cast<const float4*>(row + 4 * lane);
            float l = __shfl_up_sync(0xffffffffu, q.w, 1), r = __shfl_down_sync(0xffffffffu, q.x, 1);
            if (lane == 0) l = row[-1];
            if (lane == 31) r = row[128];
            e[ky][0] = l;
            e[ky][1] = q.x;
            e[ky][2] = q.y;
            e[ky][3] = q.z;
            e[ky][4] = q.w;
            e[ky][5] = r;
        }
    };
    auto add = [&](float (&acc)[2], const float (&e)[4][6], int kz) {
#pragma unroll
        for (int ky = 0; ky < 4; ++ky)
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int kx = 0; kx < 4; ++kx)
                    acc[m] += (wgt[kx] * wgt[ky] * wgt[kz] / 512.f) * e[ky][2 * m + kx];
    };
#pragma unroll
    for (int k = 0; k < 4; ++k) issue(k);
    float acc[2] = {0.f, 0.f}, next[2] = {0.f, 0.f}, e[4][6];
    const int co = (xc0 + 2 * lane) | ((yc0 + ty) << (I.lx - 1));
    for (int i = 0; i < NP; ++i) {
        pipe::wait_pending<1>();  // items <= i + 2 are in
        __syncthreads();          // ... for every thread; the last plane's taps are done
        resid(i);
        __syncthreads();          // the residual plane is written; x item i and b item i + 1 are free
        issue(i + 4);
        taps(e);
        if (i == 0) {
            add(acc, e, 0);
        } else if (i == 1) {
            add(acc, e, 1);
        } else if ((i & 1) == 0) {
            add(acc, e, 2);
            add(next, e, 0);
        } else {
            add(acc, e, 3);
            add(next, e, 1);
            const int o = co | ((zc0 + (i - 3) / 2) << (I.lxy - 2));
            *reinterpret_cast<float2*>(cb + o) = make_float2(acc[0], acc[1]);
            *reinterpret_cast<float2*>(cxz + o) = make_float2(0.f, 0.f);
            acc[0] = next[0];
            acc[1] = next[1];
            next[0] = next[1] = 0.f;
        }
    }
    pipe::wait_pending<0>();
}

// Trilinear prolongation-add with prolong_cell2's expressions. A thread owns
// the fine pairs x = 2t, 2t+1 of rows y = 2s, 2s+1 in planes z = 2r, 2r+1:
// fine cell 2t + 1 is the first (xcf) of coarse cell t and 2t the second
// (xnf) of coarse cell t - 1, and likewise in y and z, so the eight cells need
// the coarse values at t - 1 .. t + 1, s - 1 .. s + 1, r - 1 .. r + 1, kept in
// registers as a window of three coarse planes that moves one plane per r.
// Each fine cell takes the expression of its role (first or second in x, y
// and z) with its terms in prolong_cell2's order, and in channel mode the wall
// rows y = 0 and ny - 1 take the wall expressions: the same bits. The block's
// fine values of plane pair r (2 x 16 rows of 64 cells) and its tile of
// coarse plane r + 1 arrive in shared memory by 16-byte asynchronous copies
// issued one or two plane pairs ahead (FP64 / FP32); the sums go straight to
// memory.
template <typename T>
struct ProTile {
    static constexpr int CE = 16 / (int)sizeof(T);
    static constexpr int S = sizeof(T) == 4 ? 3 : 2;   // stages (static shared memory <= 48 KB)
    static constexpr int FROWS = 4 * kTrBY;            // 2 planes x 2 kTrBY rows
    static constexpr int FW = 64;
    static constexpr int CROWS = kTrBY + 2;
    static constexpr int CW = 32 + 2 * CE;
    static constexpr int STAGE = FROWS * FW + CROWS * CW;
};

template <typename T, int RZ>
__global__ void __launch_bounds__(32 * kTrBY) k_prolong_cols(Dims d, T* __restrict__ fine,
                                                             const T* __restrict__ coarse, int rev) {
    using P2 = typename Pair<T>::type;
    using PT = ProTile<T>;
    constexpr int CE = PT::CE;
    __shared__ __align__(16) T st[PT::S][PT::STAGE];
    const Ix2 I(d);
    const uint3 B = block_at(rev);
    const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
    const int cx = d.nx / 2, cy = d.ny / 2, cz = d.nz / 2, lcx = I.lx - 1, lcxy = I.lxy - 2;
    const int t0 = B.x * 32, s0 = B.y * kTrBY, r0 = B.z * RZ;
    const int t = t0 + lane, s = s0 + ty;
    auto crow = [&](int y) {  // coarse row y in range: clamped at channel walls, wrapped otherwise
        if (d.channel) return y < 0 ? 0 : (y > cy - 1 ? cy - 1 : y);
        return y & (cy - 1);
    };
    // item i: the fine values of plane pair r0 + i and the coarse tile of
    // plane r0 + i + 1; a commit group per item, empty past the last
    auto issue = [&](int i) {
        if (i < RZ) {
            T* dst = st[i % PT::S];
            const int r = r0 + i;
            for (int c = tid; c < PT::FROWS * (PT::FW / CE); c += 32 * kTrBY) {
                const int j = c / (PT::FW / CE), k = c - j * (PT::FW / CE);
                const int jz = j / (2 * kTrBY), jy = j - jz * (2 * kTrBY);
                pipe::cp16(dst + j * PT::FW + k * CE,
                           fine + ((2 * t0 + k * CE) | ((2 * s0 + jy) << I.lx) | ((2 * r + jz) << I.lxy)));
            }
            T* cdst = dst + PT::FROWS * PT::FW;
            const T* cpl = coarse + (((r + 1) & (cz - 1)) << lcxy);
            for (int c = tid; c < PT::CROWS * (PT::CW / CE); c += 32 * kTrBY) {
                const int j = c / (PT::CW / CE), k = c - j * (PT::CW / CE);
                const int x = (t0 - CE + k * CE) & (cx - 1);
                pipe::cp16(cdst + j * PT::CW + k * CE, cpl + (x | (crow(s0 - 1 + j) << lcx)));
            }
        }
        pipe::commit();
    };
    auto acquire = [&](int i) -> const T* {
        pipe::wait_pending<PT::S - 2>();
        __syncthreads();           // item i is in; item i - 1 is read by every thread
        issue(i + PT::S - 1);      // into item i - 1's stage
        return st[i % PT::S];
    };
#pragma unroll
    for (int i = 0; i < PT::S - 1; ++i) issue(i);
    const T a = T(27) / T(64), b = T(9) / T(64), c3 = T(3) / T(64), e = T(1) / T(64);
    const T wa = T(9) / T(16), wb = T(3) / T(16), we = T(1) / T(16);
    // interior cell of role (rx, ry, rz): 1 = first (xcf), 0 = second (xnf);
    // its base coarse cell is at offset = role in the window (x, y, z alike)
    auto cell = [&](const T (&cb)[3][3], const T (&cf)[3][3], int rx, int ry, int rz) -> T {
        const int ox = rx, oy = ry;
        const T blb = cb[oy][ox], brb = cb[oy][ox + 1], ulb = cb[oy + 1][ox], urb = cb[oy + 1][ox + 1];
        const T blf = cf[oy][ox], brf = cf[oy][ox + 1], ulf = cf[oy + 1][ox], urf = cf[oy + 1][ox + 1];
        const bool fx = rx == 1, fy = ry == 1, fz = rz == 1;
        if (fx && fy && fz) return a * blb + b * (brb + ulb + blf) + c3 * (urb + ulf + brf) + e * urf;
        if (!fx && fy && fz) return a * brb + b * (urb + blb + brf) + c3 * (ulb + blf + urf) + e * ulf;
        if (fx && !fy && fz) return a * ulb + b * (urb + blb + ulf) + c3 * (brb + blf + urf) + e * brf;
        if (!fx && !fy && fz) return a * urb + b * (brb + ulb + urf) + c3 * (blb + ulf + brf) + e * blf;
        if (fx && fy && !fz) return a * blf + b * (brf + ulf + blb) + c3 * (urf + ulb + brb) + e * urb;
        if (!fx && fy && !fz) return a * brf + b * (urf + blf + brb) + c3 * (ulf + blb + urb) + e * ulb;
        if (fx && !fy && !fz) return a * ulf + b * (urf + blf + ulb) + c3 * (brf + blb + urb) + e * brb;
        return a * urf + b * (brf + ulf + urb) + c3 * (blf + ulb + brb) + e * blb;
    };
    // channel wall cell of x role rx and z role rz, from coarse row s
    auto wall = [&](const T (&cb)[3][3], const T (&cf)[3][3], int rx, int rz) -> T {
        const int ox = rx;
        const T bl = cb[1][ox], br = cb[1][ox + 1], fl = cf[1][ox], fr = cf[1][ox + 1];
        const bool fx = rx == 1, fz = rz == 1;
        if (fx && fz) return wa * bl + wb * (br + fl) + we * fr;
        if (!fx && fz) return wa * br + wb * (bl + fr) + we * fl;
        if (fx && !fz) return wa * fl + wb * (fr + bl) + we * br;
        return wa * fr + wb * (fl + br) + we * bl;
    };
    const bool wall_lo = d.channel && s == 0, wall_hi = d.channel && s == cy - 1;
    // window: coarse planes r - 1, r, r + 1 at rows s - 1 .. s + 1, cells t - 1 .. t + 1
    T w[3][3][3];
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i)
                w[p][j][i] = coarse[((t - 1 + i) & (cx - 1)) | (crow(s - 1 + j) << lcx) |
                                    (((r0 - 1 + p) & (cz - 1)) << lcxy)];
    for (int k = 0; k < RZ; ++k) {
        const int r = r0 + k;
        const T* sf = acquire(k);
        const T* sc = sf + PT::FROWS * PT::FW;
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i) w[2][j][i] = sc[(ty + j) * PT::CW + CE + lane - 1 + i];
#pragma unroll
        for (int jz = 0; jz < 2; ++jz)
#pragma unroll
            for (int jy = 0; jy < 2; ++jy) {
                const T(&cb)[3][3] = w[jz];
                const T(&cf)[3][3] = w[jz + 1];
                T v0, v1;  // fine x = 2t (second of t - 1), 2t + 1 (first of t)
                if ((jy == 0 && wall_lo) || (jy == 1 && wall_hi)) {
                    v0 = wall(cb, cf, 0, jz);
                    v1 = wall(cb, cf, 1, jz);
                } else {
                    v0 = cell(cb, cf, 0, jy, jz);
                    v1 = cell(cb, cf, 1, jy, jz);
                }
                const P2 old = *reinterpret_cast<const P2*>(sf + (jz * 2 * kTrBY + 2 * ty + jy) * PT::FW + 2 * lane);
                P2 out;
                out.x = old.x + v0;
                out.y = old.y + v1;
                *reinterpret_cast<P2*>(fine + ((2 * t) | ((2 * s + jy) << I.lx) | ((2 * r + jz) << I.lxy))) = out;
            }
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                w[0][j][i] = w[1][j][i];
                w[1][j][i] = w[2][j][i];
            }
    }
    pipe::wait_pending<0>();
}

// Coarsest level, src/mg/solver.h:264-271: remove the mean of b, then CG
// warm-started from b with the absolute 2-norm stop. One block; the level is
// a handful of cells (one cell for a cube).
template <typename T, int TB = kRedBlock>
__device__ void coarse_cg_block(const Dims& d, T* xv, T* b, T* r, T* p, T* q, double tol, int maxit, int* status) {
    const long long N = d.ncell(), sxy = d.sxy();
    const T off = T(d.n) * T(d.n);
    __shared__ double s_val;
    auto bsum = [&](double v) {
        double a[1] = {v};
        block_sum<1, TB>(a);
        if (threadIdx.x == 0) s_val = a[0];
        __syncthreads();
        return s_val;
    };
    auto apply = [&](const T* in, long long i) {
        const int xi = (int)(i % d.nx), yi = (int)((i % sxy) / d.nx), zi = (int)(i / sxy);
        T S, c;
        // the one-cell (or one-row) levels fold self-neighbours into the diagonal
        lap_row(d, in, xi, yi, zi, S, c);
        return off * (S - c * in[i]);
    };
    double m = 0.0;
    for (long long i = threadIdx.x; i < N; i += blockDim.x) m += (double)b[i];
    m = bsum(m) / (double)N;
    for (long long i = threadIdx.x; i < N; i += blockDim.x) {
        b[i] = b[i] - T(m);
        xv[i] = b[i];
    }
    __syncthreads();
    double rr = 0.0;
    for (long long i = threadIdx.x; i < N; i += blockDim.x) {
        r[i] = b[i] - apply(xv, i);
        p[i] = r[i];
        rr += (double)r[i] * (double)r[i];
    }
    double n0 = bsum(rr);
    int it = 0;
    while (sqrt(n0) > tol) {
        if (it >= maxit || !(n0 == n0)) {
            if (threadIdx.x == 0) status[0] = 3;
            return;
        }
        double pq = 0.0;
        for (long long i = threadIdx.x; i < N; i += blockDim.x) {
            q[i] = apply(p, i);
            pq += (double)p[i] * (double)q[i];
        }
        pq = bsum(pq);
        const T alpha = T(n0 / pq);
        double n1 = 0.0;
        for (long long i = threadIdx.x; i < N; i += blockDim.x) {
            xv[i] = xv[i] + alpha * p[i];
            r[i] = r[i] - q[i] * alpha;
            n1 += (double)r[i] * (double)r[i];
        }
        n1 = bsum(n1);
        const T beta = T(n1 / n0);
        n0 = n1;
        for (long long i = threadIdx.x; i < N; i += blockDim.x) p[i] = p[i] * beta + r[i];
        __syncthreads();
        ++it;
    }
}

template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_coarse_cg(Dims d, T* __restrict__ xv, T* __restrict__ b, T* __restrict__ r,
                                                        T* __restrict__ p, T* __restrict__ q, double tol, int maxit,
                                                        int* status) {
    coarse_cg_block(d, xv, b, r, p, q, tol, maxit, status);
}

// ---------------------------------------------------------------------------
// Multigrid tail: the V-cycle below a level of at most 16^3 cells in one
// block. The coarse levels are a few thousand cells or fewer, so launching
// their ~12 kernels per level costs more than the work; here one block walks
// the same sequence (smooth, residual, restrict, zero, ..., coarsest solve,
// prolong-add, smooth) with block barriers between the phases. Every phase
// runs the per-cell function of the corresponding kernel and the coarsest
// solve is the same one-block CG, so the result equals the launch-by-launch
// V-cycle bit for bit.
// ---------------------------------------------------------------------------
// threads of the one-block tail: its phases on a 16^3 level are 2048 to 4096
// cells, so twice the reduction block size halves each phase's per-thread
// loop (1024 threads cap the registers at 64 and spill)
constexpr int kTailThreads = 512;

// cell index -> (x, y, z) for the tail's small levels (32-bit arithmetic)
__device__ __forceinline__ void tail_xyz(const Dims& d, int i, int& x, int& y, int& z) {
    const int sxy = d.nx * d.ny;
    z = i / sxy;
    const int rem = i - z * sxy;
    y = rem / d.nx;
    x = rem - y * d.nx;
}

template <typename T>
__device__ __forceinline__ void tail_sweep(const Dims& d, T* x, const T* b, int color, int t0, int ts) {
    const int hx = d.nx / 2, total = hx * d.ny * d.nz;
    for (int e = t0; e < total; e += ts) {
        const int row = e / hx, t = e - row * hx;
        const int z = row / d.ny, y = row - z * d.ny;
        const int xx = 2 * t + ((y + z + color) & 1);
        if (xx < d.nx) rbgs_cell(d, x, b, xx, y, z);
    }
}

// Power-of-two 3D levels take the shift-composed forms of the same per-cell
// functions (lap_row2, restrict_cell2, prolong_cell2: same terms, same order)
// and decode cell indices by shifts: the one-block tail is bound by the
// integer work of its phases, not by their few thousand cells' bytes.
__device__ __forceinline__ bool tail_p2(const Dims& d) {
    auto p2 = [](int v) { return (v & (v - 1)) == 0; };
    return d.nz > 1 && p2(d.nx) && p2(d.ny) && p2(d.nz);
}

template <typename T>
__device__ __forceinline__ void tail_sweep2(const Dims& d, const Ix2& I, T* x, const T* b, int color, int t0, int ts) {
    const int hx = d.nx >> 1, lhx = I.lx - 1, ly = I.lxy - I.lx, total = hx * d.ny * d.nz;
    for (int e = t0; e < total; e += ts) {
        const int t = e & (hx - 1), row = e >> lhx;
        const int y = row & I.my, z = row >> ly;
        const int xx = 2 * t + ((y + z + color) & 1);
        T S, c;
        lap_row2(d, I, x, xx, y, z, S, c);
        const int i = I.at(xx, y, z);
        const T inv = T(1) / (T(d.n) * T(d.n));
        const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
        x[i] = (S - b[i] * inv) * rc;
    }
}

// With `staged`, the levels' x, b, r (and the FP64 coarsest-level vectors)
// live in shared memory for the whole V-cycle: the top level's x and b are
// read in, the top level's x is written back (the only result the level
// above uses). Without it the phases work on the global arrays.
// CL: the same phases spread over a thread-block cluster (every CTA takes a
// share of each phase's cells; cluster barriers, whose arrive/wait release
// and acquire the phase's global writes, separate the phases). The coarsest
// solve runs in the cluster's first CTA, the same one-block CG, so the result
// is the one-block tail's, bit for bit; the levels stay in global memory (L2).
template <typename T, bool CL, int TB = kRedBlock>
__global__ void __launch_bounds__(TB, 1) k_vcycle_tail(TailLevels<T> g, int staged) {
    extern __shared__ __align__(16) unsigned char tsm[];
    // the level tables in shared memory (indexed by level: a local copy
    // would live in local memory)
    __shared__ TailLevels<T> a;
    if (threadIdx.x == 0) a = g;
    __syncthreads();
    int t0 = threadIdx.x, ts = blockDim.x;
    bool lead = true;
    if constexpr (CL) {
        namespace cg = cooperative_groups;
        const cg::cluster_group cl = cg::this_cluster();
        t0 = (int)cl.block_rank() * blockDim.x + threadIdx.x;
        ts = (int)cl.num_blocks() * blockDim.x;
        lead = cl.block_rank() == 0;
    }
    auto sync = [&]() {
        if constexpr (CL) cooperative_groups::this_cluster().sync();
        else __syncthreads();
    };
    if (!CL && staged) {
        // layout: per level x, b, r (T), then cx64, cb64, cr64, cw_p, cw_q (double)
        if (threadIdx.x == 0) {
            size_t off = 0;
            for (int l = 0; l < a.nlev; ++l) {
                const long long n = a.d[l].ncell();
                a.x[l] = (T*)(tsm + off);
                a.b[l] = a.x[l] + n;
                a.r[l] = a.b[l] + n;
                off += (size_t)3 * n * sizeof(T);
                off = (off + 15) & ~(size_t)15;
            }
            const long long nc = a.d[a.nlev - 1].ncell();
            double* dp = (double*)(tsm + off);
            a.cx64 = dp;
            a.cb64 = dp + nc;
            a.cr64 = dp + 2 * nc;
            a.cw_p = dp + 3 * nc;
            a.cw_q = dp + 4 * nc;
        }
        __syncthreads();
        const long long n0 = a.d[0].ncell();
        T* const x0 = a.x[0];
        T* const b0 = a.b[0];
        const T* const gx = g.x[0];
        const T* const gb = g.b[0];
        for (long long i = threadIdx.x; i < n0; i += blockDim.x) {
            x0[i] = gx[i];
            b0[i] = gb[i];
        }
        __syncthreads();
    }
    // per level, the dimensions and array pointers are read once into
    // registers: the level tables sit in local memory (indexed by level), and
    // through a reference every access inside the cell loops was a reload
    for (int l = 0; l + 1 < a.nlev; ++l) {
        const Dims d = a.d[l];
        T* const xl = a.x[l];
        T* const bl = a.b[l];
        T* const rl = a.r[l];
        T* const xc = a.x[l + 1];
        T* const bc = a.b[l + 1];
        const bool p2 = tail_p2(d);
        const Ix2 I(d);
        for (int j = 0; j < a.nu1; ++j) {
            for (int color = 0; color < 2; ++color) {
                if (p2) tail_sweep2(d, I, xl, bl, color, t0, ts);
                else tail_sweep(d, xl, bl, color, t0, ts);
                sync();
            }
        }
        const int n = (int)d.ncell();
        if (p2) {
            const T off = T(d.n) * T(d.n);
            for (int i = t0; i < n; i += ts) {
                const int xx = i & I.mx, yy = (i >> I.lx) & I.my, zz = i >> I.lxy;
                T S, c;
                lap_row2(d, I, xl, xx, yy, zz, S, c);
                rl[i] = bl[i] - off * (S - c * xl[i]);
            }
        } else {
            for (int i = t0; i < n; i += ts) {
                int xx, yy, zz;
                tail_xyz(d, i, xx, yy, zz);
                residual_cell(d, rl, xl, bl, xx, yy, zz);
            }
        }
        sync();
        const Dims c = a.d[l + 1];
        const int nc = (int)c.ncell();
        if (p2) {
            const int lcx = I.lx - 1, lcxy = I.lxy - 2, mcx = (d.nx >> 1) - 1, mcy = (d.ny >> 1) - 1;
            for (int i = t0; i < nc; i += ts) {
                restrict_cell2(d, I, bc, rl, i & mcx, (i >> lcx) & mcy, i >> lcxy);
                xc[i] = T(0);
            }
        } else {
            for (int i = t0; i < nc; i += ts) {
                int xx, yy, zz;
                tail_xyz(c, i, xx, yy, zz);
                restrict_cell(d, bc, rl, xx, yy, zz);
                xc[i] = T(0);
            }
        }
        sync();
    }
    if (lead) {  // block-uniform: the whole first CTA (or the one block)
        const int l = a.nlev - 1;
        const Dims& d = a.d[l];
        const long long n = d.ncell();
        if constexpr (sizeof(T) == sizeof(double)) {
            coarse_cg_block<T, TB>(d, a.x[l], a.b[l], a.r[l], a.cw_p, a.cw_q, a.tol, a.maxit, a.status);
        } else {
            for (long long i = threadIdx.x; i < n; i += blockDim.x) a.cb64[i] = (double)a.b[l][i];
            __syncthreads();
            coarse_cg_block<double, TB>(d, a.cx64, a.cb64, a.cr64, a.cw_p, a.cw_q, a.tol, a.maxit, a.status);
            __syncthreads();
            for (long long i = threadIdx.x; i < n; i += blockDim.x) a.x[l][i] = (T)a.cx64[i];
        }
    }
    sync();
    for (int l = a.nlev - 2; l >= 0; --l) {
        const Dims d = a.d[l];
        const Dims c = a.d[l + 1];
        T* const xl = a.x[l];
        T* const bl = a.b[l];
        T* const xc = a.x[l + 1];
        const bool p2 = tail_p2(d);
        const Ix2 I(d);
        const int nc = (int)c.ncell();
        if (p2) {
            const int lcx = I.lx - 1, lcxy = I.lxy - 2, mcx = (d.nx >> 1) - 1, mcy = (d.ny >> 1) - 1;
            for (int i = t0; i < nc; i += ts)
                prolong_cell2<T, true>(d, I, xl, xc, i & mcx, (i >> lcx) & mcy, i >> lcxy);
        } else {
            for (int i = t0; i < nc; i += ts) {
                int xx, yy, zz;
                tail_xyz(c, i, xx, yy, zz);
                prolong_cell<T, true>(d, xl, xc, xx, yy, zz);
            }
        }
        sync();
        for (int j = 0; j < a.nu2; ++j) {
            for (int color = 0; color < 2; ++color) {
                if (p2) tail_sweep2(d, I, xl, bl, color, t0, ts);
                else tail_sweep(d, xl, bl, color, t0, ts);
                sync();
            }
        }
    }
    if (!CL && staged) {
        const long long n0 = a.d[0].ncell();
        T* const gx = g.x[0];
        const T* const x0 = a.x[0];
        for (long long i = threadIdx.x; i < n0; i += blockDim.x) gx[i] = x0[i];
    }
}

}  // namespace

// smallest level (x extent) on which the smoother and residual take the
// batched z-column kernels (AFMIB_BATCH_MIN_NX; one cell per thread below:
// at 64^3 the batched grid is 64 blocks, and the one-cell kernels measured
// 5% faster over the coarse levels of a 256^3 V-cycle)
int batch_min_nx() {
    static const int v = [] {
        const char* e = std::getenv("AFMIB_BATCH_MIN_NX");
        return e ? std::atoi(e) : 128;
    }();
    return v;
}

template <typename T>
void launch_lap_apply(const Dims& d, T* y, const T* x, cudaStream_t s) {
    k_lap<T><<<grid3(d), dim3(BX, BY), 0, s>>>(d, y, x);
}
template <typename T>
void launch_residual(const Dims& d, T* r, const T* x, const T* b, RedScratch* sc, double* out, cudaStream_t s, int rev) {
    if (sc && out)
        k_residual_norm<T><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, r, x, b, *sc, out);
    else if (d.nz % kZU == 0 && d.nx >= batch_min_nx() && ix2_ok(d))
        k_residual_z2<T, kZU><<<dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / kZU), dim3(BX, BY), 0, s>>>(d, r, x, b,
                                                                                                          rev);
    else if (d.nz % kZU == 0 && d.nx >= batch_min_nx())
        k_residual_z<T, kZU><<<dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / kZU), dim3(BX, BY), 0, s>>>(d, r, x, b);
    else
        k_residual<T><<<grid3(d), dim3(BX, BY), 0, s>>>(d, r, x, b);
}
// The pair kernel is opt-in (AFMIB_RBGS_PAIR=1, read at every launch): at
// 256^3 its colour launches took 39.5 us against 29.9 for the scalar kernel
// (53.7 against 56.5 IB steps/s): 60 registers hold it to 4 resident blocks
// and every y-neighbour and b pair brings the other colour's value along.
// Needs full warps along x (nx >= 64) and block rows along y (ny a multiple
// of 8).
constexpr int kPairZU = 4, kPairMinB = 4;
bool rbgs_pair_ok(const Dims& d) {
    const char* e = std::getenv("AFMIB_RBGS_PAIR");
    if (!(e && e[0] == '1')) return false;
    return d.nz > 1 && d.nx >= 2 * BX && d.ny % BY == 0 && d.nz % kPairZU == 0;
}

// First colour of a sweep from x = 0 (x's contents ignored and overwritten):
// the FP32 batched kernel's own form (k_rbgs_z2b_init), elsewhere a memset of
// x and the red colour. AFMIB_INIT_SWEEP=0 takes the memset everywhere (read
// at every launch, so that a test can compare both in one process).
template <typename T>
void launch_rbgs_from_zero(const Dims& d, T* x, const T* b, cudaStream_t s, double omega, int rev) {
    const char* e = std::getenv("AFMIB_INIT_SWEEP");
    const bool off = e && e[0] == '0';
    if (d.nx < kOmegaMinNx) omega = 1.0;
    if (!off && sizeof(T) == sizeof(float) && d.nz % kZU == 0 && d.nz % kZU32 == 0 && d.nx >= batch_min_nx() &&
        ix2_ok(d) && !rbgs_pair_ok(d)) {
        const dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / kZU32);
        k_rbgs_z2b_init<T, kZU32, 6><<<g, dim3(BX, BY), 0, s>>>(d, T(omega), x, b, rev, T(0));
        return;
    }
    cudaMemsetAsync(x, 0, (size_t)d.ncell() * sizeof(T), s);
    launch_rbgs<T>(d, 0, x, b, s, omega, rev);
}

template <typename T>
void launch_rbgs(const Dims& d, int color, T* x, const T* b, cudaStream_t s, double omega, int rev) {
    if (d.nx < kOmegaMinNx) omega = 1.0;
    if (d.nz % kZU == 0 && d.nx >= batch_min_nx()) {
        dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz / kZU);
        if (ix2_ok(d)) {
            // FP32 on float pairs (opt-in, AFMIB_RBGS_PAIR=1)
            if (sizeof(T) == sizeof(float) && rbgs_pair_ok(d)) {
                const dim3 gp(d.nx / 2 / BX, d.ny / BY, d.nz / kPairZU);
                k_rbgs_pair<kPairZU, kPairMinB><<<gp, dim3(BX, BY), 0, s>>>(d, color, float(omega), (float*)x,
                                                                           (const float*)b, rev);
                return;
            }
            // FP32: kZU32 z cells per thread, registers capped for 6 resident
            // blocks (50.5 against 50.0 IB steps/s at 256^3 for eight cells
            // and 6 blocks against none; four cells: 29.5 against 30.0 us per
            // 256^3 colour, 61.1 against 60.8 steps/s; 16: spills, two:
            // 32.7 us; four cells with 8 blocks: the same as 6)
            if (sizeof(T) == sizeof(float) && d.nz % kZU32 == 0) {
                const dim3 g4(g.x, g.y, d.nz / kZU32);
                k_rbgs_z2b<T, kZU32, 6><<<g4, dim3(BX, BY), 0, s>>>(d, color, T(omega), x, b, rev);
            }
            else
                k_rbgs_z2<T, kZU><<<g, dim3(BX, BY), 0, s>>>(d, color, T(omega), x, b, rev);
        }
        else k_rbgs_z<T, kZU><<<g, dim3(BX, BY), 0, s>>>(d, color, T(omega), x, b);
        return;
    }
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz);
    k_rbgs<T><<<g, dim3(BX, BY), 0, s>>>(d, color, T(omega), x, b);
}
namespace {
int log2_exact(int v) {
    int k = 0;
    while ((1 << k) < v) ++k;
    return (1 << k) == v ? k : -1;
}
template <typename T>
void* pipe_kernel(int D, bool ch) {
    if (D == 4) return ch ? (void*)k_rbgs_pipe<T, 4, true> : (void*)k_rbgs_pipe<T, 4, false>;
    return ch ? (void*)k_rbgs_pipe<T, 2, true> : (void*)k_rbgs_pipe<T, 2, false>;
}
}  // namespace

template <typename T>
PipeCfg rbgs_pipe_cfg(const Dims& d) {
    PipeCfg c;
    const size_t row = (size_t)d.nx * sizeof(T);
    if (d.nz < 2 || d.nx < 32 || row % 16 != 0) return c;
    if (log2_exact(d.nx) < 0 || log2_exact(d.ny) < 0 || log2_exact(d.nz) < 0) return c;
    constexpr size_t kMaxSmem = 200 * 1024;
    static bool attr = false;
    if (!attr) {
        for (int dd : {4, 2})
            for (bool ch : {false, true})
                if (cudaFuncSetAttribute(pipe_kernel<T>(dd, ch), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxSmem) != cudaSuccess)
                    return c;
        attr = true;
    }
    for (int fy : {4, 2, 1}) {
        if (d.ny % fy) continue;
        for (int dd : {4, 2}) {
            const size_t smem = (size_t)(dd + 4) * (2 * fy + 6) * row;
            if (smem <= kMaxSmem) {
                c.FY = fy;
                c.D = dd;
                c.smem = smem;
                break;
            }
        }
        if (c.FY) break;
    }
    if (!c.FY) return c;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pipe_kernel<T>(c.D, d.channel != 0), kPipeThreads, c.smem);
    if (sms <= 0 || per_sm <= 0) {
        c.FY = 0;
        return c;
    }
    const int resident = sms * per_sm;
    // z chunk: the longest (least redundant halo) that still gives each
    // resident block three or more items
    const int strips = d.ny / c.FY;
    c.ZC = 0;
    for (int zc : {32, 16, 8}) {  // largest first; the smallest dividing one if none reaches 3 items
        if (d.nz % zc) continue;
        c.ZC = zc;
        if ((long long)strips * (d.nz / zc) >= 3LL * resident) break;
    }
    if (!c.ZC) c.ZC = d.nz;  // short z extents: one chunk
    const int items = strips * (d.nz / c.ZC);
    c.grid = items < resident ? items : resident;
    return c;
}

template <typename T>
void launch_rbgs_pipe(const Dims& d, const PipeCfg& c, const T* xin, T* xout, const T* b, int* err, cudaStream_t s) {
    (void)err;  // the copies are cp.async groups: no wait can time out
    const int lnx = log2_exact(d.nx), lny = log2_exact(d.ny);
    if (c.D == 4) {
        if (d.channel) k_rbgs_pipe<T, 4, true><<<c.grid, kPipeThreads, c.smem, s>>>(d, xin, xout, b, c.FY, c.ZC, lnx, lny);
        else k_rbgs_pipe<T, 4, false><<<c.grid, kPipeThreads, c.smem, s>>>(d, xin, xout, b, c.FY, c.ZC, lnx, lny);
    } else {
        if (d.channel) k_rbgs_pipe<T, 2, true><<<c.grid, kPipeThreads, c.smem, s>>>(d, xin, xout, b, c.FY, c.ZC, lnx, lny);
        else k_rbgs_pipe<T, 2, false><<<c.grid, kPipeThreads, c.smem, s>>>(d, xin, xout, b, c.FY, c.ZC, lnx, lny);
    }
}

// Column-marching transfers (k_restrict_cols, k_prolong_cols) apply to FP32
// 3D power-of-two levels with 32 | nx / 2 (64 for the restriction) and
// kTrBY | ny / 2 and 16-byte aligned fine and coarse arrays;
// AFMIB_TRANSFER_COLS=0 keeps the one-cell kernels (read at every launch, so
// that a test can compare both in one process). FP64 keeps the one-cell
// kernels: there both transfers are bound by the FP64 pipe (64 dependent FMAs
// per coarse cell, about 9 FP64 operations per prolonged cell), and the column
// kernels, with the same operations, measured 296 / 307 against 261 / 278 us
// per 256^3 launch.
static bool transfer_cols_ok(const Dims& d, const void* fine, const void* coarse) {
    if (const char* e = std::getenv("AFMIB_TRANSFER_COLS"))
        if (e[0] == '0') return false;
    return d.nz > 1 && ix2_ok(d) && (d.nx / 2) % 32 == 0 && (d.ny / 2) % kTrBY == 0 &&
           ((reinterpret_cast<uintptr_t>(fine) | reinterpret_cast<uintptr_t>(coarse)) & 15) == 0;
}
// coarse planes per thread: the largest of 8, 4, 2 that divides the coarse z
// extent and leaves at least AFMIB_TRANSFER_MIN_BLOCKS (default 1024) blocks, else 1
static int transfer_planes(const Dims& d, int bx = 32) {
    const char* e = std::getenv("AFMIB_TRANSFER_MIN_BLOCKS");
    const long long min_blocks = e ? std::atoll(e) : 1024;
    const long long cols = (long long)(d.nx / 2 / bx) * (d.ny / 2 / kTrBY);
    const int cz = d.nz / 2;
    for (int z : {8, 4, 2})
        if (cz % z == 0 && cols * (cz / z) >= min_blocks) return z;
    return 1;
}
inline dim3 transfer_grid(const Dims& d, int planes, int bx = 32) {
    return dim3(d.nx / 2 / bx, d.ny / 2 / kTrBY, d.nz / 2 / planes);
}

template <typename T>
void launch_restrict(const Dims& d, T* coarse, const T* fine, cudaStream_t s, int rev, T* zero) {
    if constexpr (sizeof(T) == sizeof(float)) {
        if (transfer_cols_ok(d, fine, coarse) && (d.nx / 2) % TrTile<T>::CX == 0 &&
            (reinterpret_cast<uintptr_t>(zero) & 15) == 0) {
            const int z = transfer_planes(d, TrTile<T>::CX);
            const dim3 g = transfer_grid(d, z, TrTile<T>::CX), b(32, kTrBY);
            if (z == 8) k_restrict_cols<T, 8><<<g, b, 0, s>>>(d, coarse, fine, rev, zero);
            else if (z == 4) k_restrict_cols<T, 4><<<g, b, 0, s>>>(d, coarse, fine, rev, zero);
            else if (z == 2) k_restrict_cols<T, 2><<<g, b, 0, s>>>(d, coarse, fine, rev, zero);
            else k_restrict_cols<T, 1><<<g, b, 0, s>>>(d, coarse, fine, rev, zero);
            return;
        }
    }
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny / 2 + BY - 1) / BY, d.nz == 1 ? 1 : d.nz / 2);
    if (d.nz > 1 && d.nx >= 2 && d.ny >= 2 && ix2_ok(d))
        k_restrict2<T><<<g, dim3(BX, BY), 0, s>>>(d, coarse, fine, rev, zero);
    else k_restrict<T><<<g, dim3(BX, BY), 0, s>>>(d, coarse, fine, zero);
}
// Fine-level residual and restriction in one pass. AFMIB_RESID_RESTRICT
// (read at every call, so that a test can compare the paths in one process):
// unset or "2": the column kernel (k_resid_restrict_cols) on FP32 levels it
// fits (3D power-of-two, 64 | nx / 2, kTrBY | ny / 2, 16-byte aligned arrays,
// nx >= AFMIB_RR_COLS_MIN_NX, default 256); "1": the ring kernel
// (k_resid_restrict2) on levels with nx >= AFMIB_RESID_RESTRICT_MIN_NX
// (default 256; on smaller levels its grid of 2 RR_T x 2 RR_T fine columns
// per block leaves SMs idle); "0": the residual and restriction kernels.
static int rr_mode(const Dims& d, size_t elem, const void* x, const void* b, const void* cb, const void* cx) {
    const char* e = std::getenv("AFMIB_RESID_RESTRICT");
    const char m = e ? e[0] : '2';
    if (m == '1') {
        const char* mn = std::getenv("AFMIB_RESID_RESTRICT_MIN_NX");
        const int min_nx = mn ? std::atoi(mn) : 256;
        return d.nz > 1 && d.nx >= min_nx && d.nx >= 2 * RR_T && d.ny >= 2 * RR_T && d.nz >= 4 && ix2_ok(d) ? 1 : 0;
    }
    if (m != '2' || elem != sizeof(float)) return 0;
    const char* mn = std::getenv("AFMIB_RR_COLS_MIN_NX");
    const int min_nx = mn ? std::atoi(mn) : 256;
    const bool aligned = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(b) |
                           reinterpret_cast<uintptr_t>(cb) | reinterpret_cast<uintptr_t>(cx)) & 15) == 0;
    return d.nz > 1 && d.nx >= min_nx && ix2_ok(d) && (d.nx / 2) % 64 == 0 && (d.ny / 2) % kTrBY == 0 && aligned
               ? 2
               : 0;
}
bool resid_restrict_fused_ok(const Dims& d, size_t elem, const void* x, const void* b, const void* cb,
                             const void* cx) {
    return rr_mode(d, elem, x, b, cb, cx) != 0;
}

void mg_kernel_attributes() {
    auto set = [](const void* f) { cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRrSmem); };
    set((const void*)k_resid_restrict_cols<8, false>);
    set((const void*)k_resid_restrict_cols<4, false>);
    set((const void*)k_resid_restrict_cols<2, false>);
    set((const void*)k_resid_restrict_cols<1, false>);
    set((const void*)k_resid_restrict_cols<8, true>);
    set((const void*)k_resid_restrict_cols<4, true>);
    set((const void*)k_resid_restrict_cols<2, true>);
    set((const void*)k_resid_restrict_cols<1, true>);
}

template <typename T>
void launch_resid_restrict(const Dims& d, T* coarse_b, T* coarse_x, const T* x, const T* b, cudaStream_t s, int rev) {
    if constexpr (sizeof(T) == sizeof(float)) {
        if (rr_mode(d, sizeof(T), x, b, coarse_b, coarse_x) == 2) {
            // coarse planes per block: the largest of 8, 4, 2 that leaves at least
            // AFMIB_RR_MIN_BLOCKS (default 512) blocks (two resident per SM)
            const char* e = std::getenv("AFMIB_RR_MIN_BLOCKS");
            const long long min_blocks = e ? std::atoll(e) : 512;
            const long long cols = (long long)(d.nx / 2 / 64) * (d.ny / 2 / kTrBY);
            const int cz = d.nz / 2;
            int z = 1;
            for (int c : {8, 4, 2})
                if (cz % c == 0 && cols * (cz / c) >= min_blocks) {
                    z = c;
                    break;
                }
            const dim3 g(d.nx / 2 / 64, d.ny / 2 / kTrBY, cz / z), blk(32, kTrBY);
            float* cbf = reinterpret_cast<float*>(coarse_b);
            float* cxf = reinterpret_cast<float*>(coarse_x);
            const float* xf = reinterpret_cast<const float*>(x);
            const float* bf = reinterpret_cast<const float*>(b);
#define AFMIB_RR_COLS(CZV)                                                                            \
    do {                                                                                              \
        if (d.channel) k_resid_restrict_cols<CZV, true><<<g, blk, kRrSmem, s>>>(d, cbf, cxf, xf, bf, rev); \
        else k_resid_restrict_cols<CZV, false><<<g, blk, kRrSmem, s>>>(d, cbf, cxf, xf, bf, rev);         \
    } while (0)
            if (z == 8) AFMIB_RR_COLS(8);
            else if (z == 4) AFMIB_RR_COLS(4);
            else if (z == 2) AFMIB_RR_COLS(2);
            else AFMIB_RR_COLS(1);
#undef AFMIB_RR_COLS
            return;
        }
    }
    // the ring kernel: coarse planes per block 8 where that still gives two
    // blocks per SM, else 2
    const int cols = (d.nx / 2 / RR_T) * (d.ny / 2 / RR_T), cz = d.nz / 2;
    if (cz % 8 == 0 && cols * (cz / 8) >= 2 * 152)
        k_resid_restrict2<T, 8><<<dim3(d.nx / 2 / RR_T, d.ny / 2 / RR_T, cz / 8), RR_THREADS, 0, s>>>(
            d, coarse_b, coarse_x, x, b, rev);
    else
        k_resid_restrict2<T, 2><<<dim3(d.nx / 2 / RR_T, d.ny / 2 / RR_T, cz / 2), RR_THREADS, 0, s>>>(
            d, coarse_b, coarse_x, x, b, rev);
}

template <typename T>
void launch_prolong_add(const Dims& d, T* fine, const T* coarse, cudaStream_t s, int rev) {
    if constexpr (sizeof(T) == sizeof(float)) {
        if (transfer_cols_ok(d, fine, coarse)) {
            // AFMIB_PROLONG_MAX_PLANES caps the planes per block (a sweep knob)
            const char* e = std::getenv("AFMIB_PROLONG_MAX_PLANES");
            int z = std::min(transfer_planes(d), e ? std::max(1, std::atoi(e)) : 8);
            while (z & (z - 1)) z &= z - 1;  // a power of two, so a divisor of the plane count
            const dim3 g = transfer_grid(d, z), b(32, kTrBY);
            if (z == 8) k_prolong_cols<T, 8><<<g, b, 0, s>>>(d, fine, coarse, rev);
            else if (z == 4) k_prolong_cols<T, 4><<<g, b, 0, s>>>(d, fine, coarse, rev);
            else if (z == 2) k_prolong_cols<T, 2><<<g, b, 0, s>>>(d, fine, coarse, rev);
            else k_prolong_cols<T, 1><<<g, b, 0, s>>>(d, fine, coarse, rev);
            return;
        }
    }
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny / 2 + BY - 1) / BY, d.nz == 1 ? 1 : d.nz / 2);
    if (d.nz > 1 && d.nx >= 2 && d.ny >= 2 && ix2_ok(d))
        k_prolong2<T, true><<<g, dim3(BX, BY), 0, s>>>(d, fine, coarse, rev);
    else k_prolong<T, true><<<g, dim3(BX, BY), 0, s>>>(d, fine, coarse);
}
template <typename T>
void launch_prolong_assign(const Dims& d, T* fine, const T* coarse, cudaStream_t s) {
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny / 2 + BY - 1) / BY, d.nz == 1 ? 1 : d.nz / 2);
    k_prolong<T, false><<<g, dim3(BX, BY), 0, s>>>(d, fine, coarse);
}
template <typename TD>
void launch_lap_defect(const Dims& d, TD* r, const double* x, const double* b, RedScratch sc, double* out, cudaStream_t s,
                       float* r_lo) {
    k_lap_defect<TD><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, r, x, b, sc, out, r_lo, lo_split());
}
void launch_lap_defect_df(const Dims& d, float* rh, float* rl, const double* x, const double* b, const double* sum,
                          double scale, RedScratch sc, double* out, cudaStream_t s) {
    k_lap_defect_df<<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, rh, rl, x, b, sum, scale, sc, out);
}
void launch_lap_update_df(const Dims& d, double* x, const float* e, float* rh, float* rl, RedScratch sc, double* out,
                          cudaStream_t s) {
    constexpr int ZU = 2;
    const char* g = std::getenv("AFMIB_UPDATE_DF_GENERIC");
    if (d.nz > 1 && d.nz % ZU == 0 && ix2_ok(d) && !(g && g[0] == '1')) {
        const int gx = (d.nx + kRBX - 1) / kRBX, gy = (d.ny + kRBY - 1) / kRBY;
        int gz = d.nz / ZU;
        if ((long long)gx * gy * gz > kMaxRedBlocks) gz = std::max(1, kMaxRedBlocks / (gx * gy));
        k_lap_update_df2<ZU, kUpdateMinBlocks><<<dim3(gx, gy, gz), dim3(kRBX, kRBY), 0, s>>>(d, x, e, rh, rl, sc, out);
        return;
    }
    k_lap_update_df<<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, x, e, rh, rl, sc, out);
}
bool launch_lap_defect_bfp(const Dims& d, float* r, const double* x, const double* b, RedScratch sc, double* out,
                           cudaStream_t s) {
    int k = 0;
    while ((1 << k) < d.n) ++k;
    if ((1 << k) != d.n || 2 * k > 126) return false;  // n must be a power of two
    k_lap_defect_bfp<<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, 2 * k, r, x, b, sc, out);
    return true;
}
template void launch_lap_defect<float>(const Dims&, float*, const double*, const double*, RedScratch, double*,
                                       cudaStream_t, float*);

template <typename T>
void launch_vcycle_tail(const TailLevels<T>& a, cudaStream_t s, int cluster) {
    if (cluster > 1) {
        if (cluster > 8) {
            static bool np = false;
            if (!np)
                np = cudaFuncSetAttribute(k_vcycle_tail<T, true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                     cudaSuccess;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cluster);
        cfg.blockDim = dim3(kRedBlock);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cluster;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_vcycle_tail<T, true>, a, 0);  // errors reach the caller's cudaGetLastError
        return;
    }
    // shared-memory staging when the levels fit
    size_t bytes = 0;
    for (int l = 0; l < a.nlev; ++l) {
        bytes += (size_t)3 * a.d[l].ncell() * sizeof(T);
        bytes = (bytes + 15) & ~(size_t)15;
    }
    bytes += (size_t)5 * a.d[a.nlev - 1].ncell() * sizeof(double);
    // one block of kTailThreads (AFMIB_TAIL_THREADS=256 or 1024 instead):
    // the phases are per-cell and the coarsest CG sums the same cells in the
    // same order, so the block size does not change the result
    constexpr size_t kMax = 160 * 1024;
    // read at every launch (graphs capture it once), so that a test can compare block sizes
    const int threads = [] {
        const char* e = std::getenv("AFMIB_TAIL_THREADS");
        const int v = e ? std::atoi(e) : kTailThreads;
        return v == 1024 || v == kRedBlock ? v : kTailThreads;
    }();
    static bool attr = false, attr_big = false, attr_1k = false;
    if (threads == kTailThreads) {
        if (!attr_big)
            attr_big = cudaFuncSetAttribute(k_vcycle_tail<T, false, kTailThreads>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMax) == cudaSuccess;
        if (attr_big && bytes <= kMax) k_vcycle_tail<T, false, kTailThreads><<<1, kTailThreads, bytes, s>>>(a, 1);
        else k_vcycle_tail<T, false, kTailThreads><<<1, kTailThreads, 0, s>>>(a, 0);
        return;
    }
    if (threads == 1024) {
        if (!attr_1k)
            attr_1k = cudaFuncSetAttribute(k_vcycle_tail<T, false, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)kMax) == cudaSuccess;
        if (attr_1k && bytes <= kMax) k_vcycle_tail<T, false, 1024><<<1, 1024, bytes, s>>>(a, 1);
        else k_vcycle_tail<T, false, 1024><<<1, 1024, 0, s>>>(a, 0);
        return;
    }
    if (!attr)
        attr = cudaFuncSetAttribute(k_vcycle_tail<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMax) ==
               cudaSuccess;
    if (attr && bytes <= kMax) k_vcycle_tail<T, false><<<1, kRedBlock, bytes, s>>>(a, 1);
    else k_vcycle_tail<T, false><<<1, kRedBlock, 0, s>>>(a, 0);
}

int vcycle_tail_cluster_max() {
    for (int cs : {16, 8, 4}) {
        if (cs > 8 && cudaFuncSetAttribute(k_vcycle_tail<float, true>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                                           1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(kRedBlock);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_vcycle_tail<float, true>, &cfg) == cudaSuccess && n > 0) return cs;
        cudaGetLastError();
    }
    return 1;
}
template <typename T>
void launch_coarse_solve(const Dims& d, T* x, T* b, T* r, T* p, T* q, double tol, int maxit, int* status, cudaStream_t s) {
    k_coarse_cg<T><<<1, kRedBlock, 0, s>>>(d, x, b, r, p, q, tol, maxit, status);
}

#define AFMIB_MG_INST(T)                                                                                 \
    template void launch_lap_apply<T>(const Dims&, T*, const T*, cudaStream_t);                          \
    template void launch_residual<T>(const Dims&, T*, const T*, const T*, RedScratch*, double*, cudaStream_t, int); \
    template void launch_rbgs<T>(const Dims&, int, T*, const T*, cudaStream_t, double, int);                        \
    template void launch_rbgs_from_zero<T>(const Dims&, T*, const T*, cudaStream_t, double, int);                  \
    template PipeCfg rbgs_pipe_cfg<T>(const Dims&);                                                      \
    template void launch_rbgs_pipe<T>(const Dims&, const PipeCfg&, const T*, T*, const T*, int*, cudaStream_t); \
    template void launch_restrict<T>(const Dims&, T*, const T*, cudaStream_t, int, T*);                     \
    template void launch_prolong_add<T>(const Dims&, T*, const T*, cudaStream_t, int);                      \
    template void launch_resid_restrict<T>(const Dims&, T*, T*, const T*, const T*, cudaStream_t, int);      \
    template void launch_prolong_assign<T>(const Dims&, T*, const T*, cudaStream_t);                     \
    template void launch_coarse_solve<T>(const Dims&, T*, T*, T*, T*, T*, double, int, int*, cudaStream_t);    \
    template void launch_vcycle_tail<T>(const TailLevels<T>&, cudaStream_t, int);

AFMIB_MG_INST(double)
AFMIB_MG_INST(float)

}  // namespace afmib
