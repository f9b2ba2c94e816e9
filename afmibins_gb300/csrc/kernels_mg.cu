// Geometric multigrid pieces for the pressure projection (src/mg/solver.h,
// src/mg/laplacian.h): red-black Gauss–Seidel in place of the reference's
// lexicographic CSR sweep, the reference's full-weighting restriction and
// trilinear prolongation, and a one-block CG for the coarsest level.
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
__device__ __forceinline__ void lap_row(const Dims& d, const T* __restrict__ x, int xi, int yi, int zi, T& S, T& c) {
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

template <typename T>
__global__ void k_residual(Dims d, T* __restrict__ r, const T* __restrict__ xv, const T* __restrict__ b) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= d.nx || y >= d.ny) return;
    T S, c;
    lap_row(d, xv, x, y, z, S, c);
    const long long i = lin(d, x, y, z);
    const T off = T(d.n) * T(d.n);
    r[i] = b[i] - off * (S - c * xv[i]);
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
template <typename TD>
__global__ void __launch_bounds__(kRedBlock) k_lap_defect(Dims d, TD* __restrict__ r, const double* __restrict__ xv,
                                                         const double* __restrict__ b, RedScratch sc, double* out) {
    const int xi = blockIdx.x * kRBX + threadIdx.x, yi = blockIdx.y * kRBY + threadIdx.y;
    const double off = double(d.n) * double(d.n);
    TD acc = TD(0);
    if (xi < d.nx && yi < d.ny)
#pragma unroll 2
        for (int zi = blockIdx.z; zi < d.nz; zi += gridDim.z) {
            double S, c;
            lap_row(d, xv, xi, yi, zi, S, c);
            const long long i = lin(d, xi, yi, zi);
            const TD ri = TD(b[i] - off * (S - c * xv[i]));
            r[i] = ri;
            acc += ri * ri;
        }
    double a[1] = {(double)acc};
    grid_sum<1>(a, sc, out);
}

// One colour of red-black Gauss–Seidel: x_i = (b_i - n^2 S) / (-c n^2).
template <typename T>
__global__ void k_rbgs(Dims d, int color, T* __restrict__ xv, const T* __restrict__ b) {
    const int y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    const int x = 2 * (blockIdx.x * BX + threadIdx.x) + ((y + z + color) & 1);
    if (x >= d.nx || y >= d.ny) return;
    T S, c;
    lap_row(d, xv, x, y, z, S, c);
    const long long i = lin(d, x, y, z);
    const T inv = T(1) / (T(d.n) * T(d.n));
    const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
    xv[i] = (S - b[i] * inv) * rc;
}

// ---------------------------------------------------------------------------
// Tile-fused red-black sweep: one launch performs the red half sweep and the
// black half sweep, reading x and b once and writing x once (3N words per full
// sweep instead of the per-colour kernels' ~4.6N). A block owns an FX x FY
// (x, y) tile and a chunk of FZ planes; it marches k along z with a ring of
// four planes of x (tile + 2-cell halo) in shared memory: the red cells of
// plane k are updated on the tile + 1-cell halo (they need the old black
// values), then the black cells of plane k-1 on the tile (they need the new
// red values of planes k-2, k-1, k), and plane k-1 is written out. The sweep
// is out of place (xin -> xout): blocks read only old values, recompute the
// red halo redundantly from them, and the result equals the two per-colour
// launches cell for cell (same arithmetic, same summation order).
// ---------------------------------------------------------------------------
constexpr int FX = 32, FY = 16, FZ = 16;
constexpr int HX = FX + 4, HY = FY + 4;  // x ring planes with halo 2

template <typename T>
__global__ void __launch_bounds__(FX * FY) k_rbgs_fused(Dims d, const T* __restrict__ xin, T* __restrict__ xout,
                                                        const T* __restrict__ b) {
    __shared__ T ring[4][HY][HX];
    __shared__ T bpl[2][FY + 2][FX + 2];
    const int tid = threadIdx.x + FX * threadIdx.y;
    const int x0 = blockIdx.x * FX, y0 = blockIdx.y * FY, z0 = blockIdx.z * FZ;
    const int zend = min(z0 + FZ, d.nz);
    const T inv = T(1) / (T(d.n) * T(d.n));
    // load plane z (wrapped) of x into ring slot: tile + halo 2
    auto load_x = [&](int z) {
        const int zz = wrapi(z, d.nz);
        T(*pl)[HX] = ring[((z % 4) + 4) % 4];
        for (int e = tid; e < HX * HY; e += FX * FY) {
            const int hx = e % HX, hy = e / HX;
            const int gx = wrapi(x0 + hx - 2, d.nx);
            int gy = y0 + hy - 2;
            T val = T(0);
            if (d.channel) {
                if (gy >= 0 && gy < d.ny) val = xin[lin(d, gx, gy, zz)];
            } else {
                val = xin[lin(d, gx, wrapi(gy, d.ny), zz)];
            }
            pl[hy][hx] = val;
        }
    };
    auto load_b = [&](int z) {
        const int zz = wrapi(z, d.nz);
        T(*pl)[FX + 2] = bpl[((z % 2) + 2) % 2];
        for (int e = tid; e < (FX + 2) * (FY + 2); e += FX * FY) {
            const int hx = e % (FX + 2), hy = e / (FX + 2);
            const int gx = wrapi(x0 + hx - 1, d.nx);
            int gy = y0 + hy - 1;
            T val = T(0);
            if (d.channel) {
                if (gy >= 0 && gy < d.ny) val = b[lin(d, gx, gy, zz)];
            } else {
                val = b[lin(d, gx, wrapi(gy, d.ny), zz)];
            }
            pl[hy][hx] = val;
        }
    };
    // Gauss-Seidel update of the cell at ring coordinates (hx, hy) of plane z
    auto update = [&](int z, int hx, int hy, T bval) {
        T(*c0)[HX] = ring[((z % 4) + 4) % 4];
        T(*cm)[HX] = ring[(((z - 1) % 4) + 4) % 4];
        T(*cp)[HX] = ring[(((z + 1) % 4) + 4) % 4];
        T S = (c0[hy][hx - 1] + c0[hy][hx + 1]) + (cm[hy][hx] + cp[hy][hx]);
        T c = T(6);
        if (d.channel) {
            const int gy = y0 + hy - 2;
            if (gy > 0) S += c0[hy - 1][hx]; else c -= T(1);
            if (gy < d.ny - 1) S += c0[hy + 1][hx]; else c -= T(1);
        } else {
            S += c0[hy - 1][hx] + c0[hy + 1][hx];
        }
        const T rc = (c == T(6)) ? T(1.0 / 6.0) : ((c == T(5)) ? T(1.0 / 5.0) : (c == T(4) ? T(0.25) : T(1) / c));
        c0[hy][hx] = (S - bval * inv) * rc;
    };
    load_x(z0 - 2);
    load_x(z0 - 1);
    load_x(z0);
    for (int k = z0 - 1; k <= zend; ++k) {
        load_x(k + 1);
        load_b(k);
        __syncthreads();
        // red cells of plane k on the tile + 1-cell halo
        {
            T(*bk)[FX + 2] = bpl[((k % 2) + 2) % 2];
            for (int e = tid; e < (FX + 2) * (FY + 2); e += FX * FY) {
                const int ex = e % (FX + 2), ey = e / (FX + 2);
                const int gx = x0 + ex - 1, gy = y0 + ey - 1;
                if (d.channel && (gy < 0 || gy >= d.ny)) continue;
                if (((wrapi(gx, d.nx) + wrapi(gy, d.ny) + wrapi(k, d.nz)) & 1) != 0) continue;
                update(k, ex + 1, ey + 1, bk[ey][ex]);
            }
        }
        __syncthreads();
        // black cells of plane k-1 on the tile, then write plane k-1
        if (k - 1 >= z0 && k - 1 < zend) {
            const int zb = k - 1;
            T(*bk)[FX + 2] = bpl[((zb % 2) + 2) % 2];
            const int lx = threadIdx.x, ly = threadIdx.y;
            const int gx = x0 + lx, gy = y0 + ly;
            if (gx < d.nx && gy < d.ny && (((gx + gy + zb) & 1) != 0)) update(zb, lx + 2, ly + 2, bk[ly + 1][lx + 1]);
            __syncthreads();
            if (gx < d.nx && gy < d.ny) xout[lin(d, gx, gy, zb)] = ring[((zb % 4) + 4) % 4][ly + 2][lx + 2];
        }
        __syncthreads();
    }
}

// Full weighting, src/mg/solver.h:153-181: 64 taps (1,3,3,1)^3/512 around the
// coarse cell; y clamps at the channel walls, wraps in periodic mode.
template <typename T>
__global__ void k_restrict(Dims d, T* __restrict__ coarse, const T* __restrict__ fine) {
    const int cx = d.nx / 2, cy = d.ny / 2, cz = d.nz / 2;
    const int xc = blockIdx.x * BX + threadIdx.x, yc = blockIdx.y * BY + threadIdx.y, zc = blockIdx.z;
    if (xc >= cx || yc >= cy) return;
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

// Trilinear prolongation (27,9,3,1)/64, src/mg/solver.h:71-151. One thread per
// coarse cell writes the eight fine cells between it and its +1 neighbours;
// in channel mode the wall rows take the bilinear (9,3,1)/16 weights.
template <typename T, bool ADD>
__global__ void k_prolong(Dims d, T* __restrict__ fine, const T* __restrict__ coarse) {
    const int cx = d.nx / 2, cy = d.ny / 2, cz = d.nz / 2;
    const int xc = blockIdx.x * BX + threadIdx.x, yc = blockIdx.y * BY + threadIdx.y, zc = blockIdx.z;
    if (xc >= cx || yc >= cy) return;
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

// Coarsest level, src/mg/solver.h:264-271: remove the mean of b, then CG
// warm-started from b with the absolute 2-norm stop. One block; the level is
// a handful of cells (one cell for a cube).
template <typename T>
__global__ void __launch_bounds__(kRedBlock) k_coarse_cg(Dims d, T* __restrict__ xv, T* __restrict__ b, T* __restrict__ r,
                                                        T* __restrict__ p, T* __restrict__ q, double tol, int maxit,
                                                        int* status) {
    const long long N = d.ncell(), sxy = d.sxy();
    const T off = T(d.n) * T(d.n);
    __shared__ double s_val;
    auto bsum = [&](double v) {
        double a[1] = {v};
        block_sum<1>(a);
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

}  // namespace

template <typename T>
void launch_lap_apply(const Dims& d, T* y, const T* x, cudaStream_t s) {
    k_lap<T><<<grid3(d), dim3(BX, BY), 0, s>>>(d, y, x);
}
template <typename T>
void launch_residual(const Dims& d, T* r, const T* x, const T* b, RedScratch* sc, double* out, cudaStream_t s) {
    if (sc && out)
        k_residual_norm<T><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, r, x, b, *sc, out);
    else
        k_residual<T><<<grid3(d), dim3(BX, BY), 0, s>>>(d, r, x, b);
}
template <typename T>
void launch_rbgs(const Dims& d, int color, T* x, const T* b, cudaStream_t s) {
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz);
    k_rbgs<T><<<g, dim3(BX, BY), 0, s>>>(d, color, x, b);
}
template <typename T>
void launch_rbgs_fused(const Dims& d, const T* xin, T* xout, const T* b, cudaStream_t s) {
    dim3 g((d.nx + FX - 1) / FX, (d.ny + FY - 1) / FY, (d.nz + FZ - 1) / FZ);
    k_rbgs_fused<T><<<g, dim3(FX, FY), 0, s>>>(d, xin, xout, b);
}
bool rbgs_fused_ok(const Dims& d) { return d.nx >= FX && d.ny >= FY && d.nz >= FZ; }

template <typename T>
void launch_restrict(const Dims& d, T* coarse, const T* fine, cudaStream_t s) {
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny / 2 + BY - 1) / BY, d.nz == 1 ? 1 : d.nz / 2);
    k_restrict<T><<<g, dim3(BX, BY), 0, s>>>(d, coarse, fine);
}
template <typename T>
void launch_prolong_add(const Dims& d, T* fine, const T* coarse, cudaStream_t s) {
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny / 2 + BY - 1) / BY, d.nz == 1 ? 1 : d.nz / 2);
    k_prolong<T, true><<<g, dim3(BX, BY), 0, s>>>(d, fine, coarse);
}
template <typename T>
void launch_prolong_assign(const Dims& d, T* fine, const T* coarse, cudaStream_t s) {
    dim3 g((d.nx / 2 + BX - 1) / BX, (d.ny / 2 + BY - 1) / BY, d.nz == 1 ? 1 : d.nz / 2);
    k_prolong<T, false><<<g, dim3(BX, BY), 0, s>>>(d, fine, coarse);
}
template <typename TD>
void launch_lap_defect(const Dims& d, TD* r, const double* x, const double* b, RedScratch sc, double* out, cudaStream_t s) {
    k_lap_defect<TD><<<red_grid3(d.nx, d.ny, d.nz), dim3(kRBX, kRBY), 0, s>>>(d, r, x, b, sc, out);
}
template void launch_lap_defect<float>(const Dims&, float*, const double*, const double*, RedScratch, double*,
                                       cudaStream_t);

template <typename T>
void launch_coarse_solve(const Dims& d, T* x, T* b, T* r, T* p, T* q, double tol, int maxit, int* status, cudaStream_t s) {
    k_coarse_cg<T><<<1, kRedBlock, 0, s>>>(d, x, b, r, p, q, tol, maxit, status);
}

#define AFMIB_MG_INST(T)                                                                                 \
    template void launch_lap_apply<T>(const Dims&, T*, const T*, cudaStream_t);                          \
    template void launch_residual<T>(const Dims&, T*, const T*, const T*, RedScratch*, double*, cudaStream_t); \
    template void launch_rbgs<T>(const Dims&, int, T*, const T*, cudaStream_t);                          \
    template void launch_rbgs_fused<T>(const Dims&, const T*, T*, const T*, cudaStream_t);               \
    template void launch_restrict<T>(const Dims&, T*, const T*, cudaStream_t);                           \
    template void launch_prolong_add<T>(const Dims&, T*, const T*, cudaStream_t);                        \
    template void launch_prolong_assign<T>(const Dims&, T*, const T*, cudaStream_t);                     \
    template void launch_coarse_solve<T>(const Dims&, T*, T*, T*, T*, T*, double, int, int*, cudaStream_t);

AFMIB_MG_INST(double)
AFMIB_MG_INST(float)

}  // namespace afmib
