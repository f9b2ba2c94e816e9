// Adjoint kernels of the immersed-boundary step (periodic domain).
//
// The reference has no adjoint. These are the transposes of the forward
// kernels' derivatives, used by the reverse pass in solver.cu:
//  - advection: N(u) is quadratic in u (src/ns/solver.h:142-236); its
//    Jacobian transposed acts on an adjoint lam = (lu, lv, lw) as a gather
//    over the six flux terms that touch each face;
//  - marker positions: derivatives of the cosine 4-point weights
//    (src/ib/grid.h:51-55), d/ds [(1-S)/4, (1+C)/4, (1+S)/4, (1-C)/4] =
//    pi/8 [-C, -S, C, S] with s = X n, S = sin(pi t/2), C = cos(pi t/2);
//  - springs: G = k K X with K the (symmetric) neighbour-difference operator.
#include "kernels_adjoint.h"

namespace afmib {

namespace {

constexpr int BX = 32, BY = 8;
inline dim3 grid3(const Dims& d) { return dim3((d.nx + BX - 1) / BX, (d.ny + BY - 1) / BY, d.nz); }

struct Ix {
    Dims d;
    __device__ long long operator()(int x, int y, int z) const {
        return lin(d, wrapi(x, d.nx), wrapi(y, d.ny), wrapi(z, d.nz));
    }
};

// Flux adjoints at index (x, y, z): L_UU = n (lu[j-x] - lu[j]) etc.
__device__ __forceinline__ double LUU(const Ix& I, const double* lu, double n, int x, int y, int z) {
    return n * (lu[I(x - 1, y, z)] - lu[I(x, y, z)]);
}
__device__ __forceinline__ double LVV(const Ix& I, const double* lv, double n, int x, int y, int z) {
    return n * (lv[I(x, y - 1, z)] - lv[I(x, y, z)]);
}
__device__ __forceinline__ double LWW(const Ix& I, const double* lw, double n, int x, int y, int z) {
    return n * (lw[I(x, y, z - 1)] - lw[I(x, y, z)]);
}
__device__ __forceinline__ double LUV(const Ix& I, const double* lu, const double* lv, double n, int x, int y, int z) {
    return n * (lu[I(x, y - 1, z)] - lu[I(x, y, z)]) + n * (lv[I(x - 1, y, z)] - lv[I(x, y, z)]);
}
__device__ __forceinline__ double LUW(const Ix& I, const double* lu, const double* lw, double n, int x, int y, int z) {
    return n * (lu[I(x, y, z - 1)] - lu[I(x, y, z)]) + n * (lw[I(x - 1, y, z)] - lw[I(x, y, z)]);
}
__device__ __forceinline__ double LVW(const Ix& I, const double* lv, const double* lw, double n, int x, int y, int z) {
    return n * (lv[I(x, y, z - 1)] - lv[I(x, y, z)]) + n * (lw[I(x, y - 1, z)] - lw[I(x, y, z)]);
}

// out = N'(u)^T lam, accumulated (out += ...) when acc != 0
__global__ void k_advect_adjoint(Dims d, double* __restrict__ ou, double* __restrict__ ov, double* __restrict__ ow,
                                 const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ w,
                                 const double* __restrict__ lu, const double* __restrict__ lv,
                                 const double* __restrict__ lw, int acc) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
    if (x >= d.nx || y >= d.ny) return;
    const Ix I{d};
    const double n = d.n;
    // averages used by the flux products at index j
    auto qUU = [&](int a, int b, int c) { return 0.5 * (u[I(a, b, c)] + u[I(a - 1, b, c)]); };
    auto qVV = [&](int a, int b, int c) { return 0.5 * (v[I(a, b, c)] + v[I(a, b - 1, c)]); };
    auto qWW = [&](int a, int b, int c) { return 0.5 * (w[I(a, b, c)] + w[I(a, b, c - 1)]); };
    auto quy = [&](int a, int b, int c) { return 0.5 * (u[I(a, b, c)] + u[I(a, b - 1, c)]); };  // u in UV
    auto qvx = [&](int a, int b, int c) { return 0.5 * (v[I(a, b, c)] + v[I(a - 1, b, c)]); };  // v in UV
    auto quz = [&](int a, int b, int c) { return 0.5 * (u[I(a, b, c)] + u[I(a, b, c - 1)]); };  // u in UW
    auto qwx = [&](int a, int b, int c) { return 0.5 * (w[I(a, b, c)] + w[I(a - 1, b, c)]); };  // w in UW
    auto qvz = [&](int a, int b, int c) { return 0.5 * (v[I(a, b, c)] + v[I(a, b, c - 1)]); };  // v in VW
    auto qwy = [&](int a, int b, int c) { return 0.5 * (w[I(a, b, c)] + w[I(a, b - 1, c)]); };  // w in VW
    // UU(j) = q^2 -> dUU/du[j] = dUU/du[j-x] = q; UV(j) = qu qv -> d/du = qv/2 ...
    const double gu = LUU(I, lu, n, x, y, z) * qUU(x, y, z) + LUU(I, lu, n, x + 1, y, z) * qUU(x + 1, y, z) +
                      0.5 * (LUV(I, lu, lv, n, x, y, z) * qvx(x, y, z) + LUV(I, lu, lv, n, x, y + 1, z) * qvx(x, y + 1, z)) +
                      0.5 * (LUW(I, lu, lw, n, x, y, z) * qwx(x, y, z) + LUW(I, lu, lw, n, x, y, z + 1) * qwx(x, y, z + 1));
    const double gv = LVV(I, lv, n, x, y, z) * qVV(x, y, z) + LVV(I, lv, n, x, y + 1, z) * qVV(x, y + 1, z) +
                      0.5 * (LUV(I, lu, lv, n, x, y, z) * quy(x, y, z) + LUV(I, lu, lv, n, x + 1, y, z) * quy(x + 1, y, z)) +
                      0.5 * (LVW(I, lv, lw, n, x, y, z) * qwy(x, y, z) + LVW(I, lv, lw, n, x, y, z + 1) * qwy(x, y, z + 1));
    const double gw = LWW(I, lw, n, x, y, z) * qWW(x, y, z) + LWW(I, lw, n, x, y, z + 1) * qWW(x, y, z + 1) +
                      0.5 * (LUW(I, lu, lw, n, x, y, z) * quz(x, y, z) + LUW(I, lu, lw, n, x + 1, y, z) * quz(x + 1, y, z)) +
                      0.5 * (LVW(I, lv, lw, n, x, y, z) * qvz(x, y, z) + LVW(I, lv, lw, n, x, y + 1, z) * qvz(x, y + 1, z));
    const long long i = lin(d, x, y, z);
    if (acc) {
        ou[i] += gu;
        ov[i] += gv;
        ow[i] += gw;
    } else {
        ou[i] = gu;
        ov[i] = gv;
        ow[i] = gw;
    }
}

// weights and their s-derivatives for one axis: t = frac(s - off)
__device__ __forceinline__ void weights4(double s, double off, int& base, double w[4], double dw[4]) {
    const double t = s - off;
    const double ft = floor(t);
    const double fr = t - ft;
    base = (int)ft - 1;
    double S, C;
    sincospi(0.5 * fr, &S, &C);
    w[0] = 0.25 * (1.0 - S);
    w[1] = 0.25 * (1.0 + C);
    w[2] = 0.25 * (1.0 + S);
    w[3] = 0.25 * (1.0 - C);
    const double q = 0.125 * 3.14159265358979323846;
    dw[0] = -q * C;
    dw[1] = -q * S;
    dw[2] = q * C;
    dw[3] = q * S;
}

// gX[k][a] += scale * sum_c g[c][k] * sum_faces d/dX_a (phi/n)^3_c * F_c(face)
__global__ void k_marker_grad(Dims d, int M, const double* __restrict__ X, const double* __restrict__ g,
                              const double* __restrict__ Fu, const double* __restrict__ Fv,
                              const double* __restrict__ Fw, double scale, double* __restrict__ gX) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    const int ext[3] = {d.nx, d.ny, d.nz};
    double out[3] = {0.0, 0.0, 0.0};
    for (int comp = 0; comp < 3; ++comp) {
        const double gc = g[(size_t)comp * M + k];
        if (gc == 0.0) continue;
        const double* F = comp == 0 ? Fu : (comp == 1 ? Fv : Fw);
        int base[3];
        double w[3][4], dw[3][4];
        for (int a = 0; a < 3; ++a) weights4(X[3 * k + a] * d.n, a == comp ? 0.0 : 0.5, base[a], w[a], dw[a]);
        double sx = 0, sy = 0, sz = 0;
        for (int mz = 0; mz < 4; ++mz)
            for (int my = 0; my < 4; ++my)
                for (int mx = 0; mx < 4; ++mx) {
                    const double f = F[lin(d, wrapi(base[0] + mx, ext[0]), wrapi(base[1] + my, ext[1]),
                                           wrapi(base[2] + mz, ext[2]))];
                    sx += dw[0][mx] * w[1][my] * w[2][mz] * f;
                    sy += w[0][mx] * dw[1][my] * w[2][mz] * f;
                    sz += w[0][mx] * w[1][my] * dw[2][mz] * f;
                }
        out[0] += gc * sx;
        out[1] += gc * sy;
        out[2] += gc * sz;
    }
    // d/dX = n d/ds
    gX[3 * k + 0] += scale * d.n * out[0];
    gX[3 * k + 1] += scale * d.n * out[1];
    gX[3 * k + 2] += scale * d.n * out[2];
}

// Springs transpose: gX[i] += k * (K^T lamG)[i] for symmetric neighbour lists,
// and per-marker partials of d/dk = sum_i lamG_i . (K X)_i
__global__ void k_springs_adjoint(int M, const double* __restrict__ X, const int* __restrict__ ns,
                                  const int* __restrict__ ni, double kspring, const double* __restrict__ lamG,
                                  double* __restrict__ gX, double* __restrict__ dk_part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    double kx[3] = {0, 0, 0}, kt[3] = {0, 0, 0};
    const double li[3] = {lamG[i], lamG[M + i], lamG[2 * M + i]};
    for (int e = ns[i]; e < ns[i + 1]; ++e) {
        const int j = ni[e];
        for (int a = 0; a < 3; ++a) {
            kx[a] += X[3 * j + a] - X[3 * i + a];
            // (K^T lam)_i = sum_{j in N(i)} lam_j - deg_i lam_i when N is symmetric
            kt[a] += lamG[(size_t)a * M + j] - li[a];
        }
    }
    for (int a = 0; a < 3; ++a) gX[3 * i + a] += kspring * kt[a];
    dk_part[i] = li[0] * kx[0] + li[1] * kx[1] + li[2] * kx[2];
}

// Bending part of the marker-force adjoint: gX += -kb L (L lamG) (L
// symmetric), in two passes through Z = L lamG (stored like lamG).
__global__ void k_lap_soa(int M, const double* __restrict__ lam, const int* __restrict__ ns,
                          const int* __restrict__ ni, double* __restrict__ Z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    for (int a = 0; a < 3; ++a) {
        const double li = lam[(size_t)a * M + i];
        double z = 0;
        for (int e = ns[i]; e < ns[i + 1]; ++e) z += lam[(size_t)a * M + ni[e]] - li;
        Z[(size_t)a * M + i] = z;
    }
}
__global__ void k_bend_adjoint(int M, const double* __restrict__ Z, const int* __restrict__ ns,
                               const int* __restrict__ ni, double kb, double* __restrict__ gX) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    for (int a = 0; a < 3; ++a) {
        const double zi = Z[(size_t)a * M + i];
        double b = 0;
        for (int e = ns[i]; e < ns[i + 1]; ++e) b += Z[(size_t)a * M + ni[e]] - zi;
        gX[3 * i + a] += -kb * b;
    }
}

}  // namespace

void launch_bending_adjoint(int M, const int* ns, const int* ni, double kb, const double* lamG, double* Z, double* gX,
                            cudaStream_t s) {
    if (M <= 0) return;
    k_lap_soa<<<(M + 255) / 256, 256, 0, s>>>(M, lamG, ns, ni, Z);
    k_bend_adjoint<<<(M + 255) / 256, 256, 0, s>>>(M, Z, ns, ni, kb, gX);
}

void launch_advect_adjoint(const Dims& d, double* ou, double* ov, double* ow, const double* u, const double* v,
                           const double* w, const double* lu, const double* lv, const double* lw, int acc,
                           cudaStream_t s) {
    k_advect_adjoint<<<grid3(d), dim3(BX, BY), 0, s>>>(d, ou, ov, ow, u, v, w, lu, lv, lw, acc);
}

void launch_marker_grad(const Dims& d, int M, const double* X, const double* g, const double* Fu, const double* Fv,
                        const double* Fw, double scale, double* gX, cudaStream_t s) {
    if (M > 0) k_marker_grad<<<(M + 127) / 128, 128, 0, s>>>(d, M, X, g, Fu, Fv, Fw, scale, gX);
}

void launch_springs_adjoint(int M, const double* X, const int* ns, const int* ni, double kspring, const double* lamG,
                            double* gX, double* dk_part, cudaStream_t s) {
    if (M > 0) k_springs_adjoint<<<(M + 255) / 256, 256, 0, s>>>(M, X, ns, ni, kspring, lamG, gX, dk_part);
}

}  // namespace afmib

namespace afmib {
namespace {
// soa[c*M + k] = c0 * aos[3k + c]
__global__ void k_aos_to_soa(int M, const double* __restrict__ aos, double* __restrict__ soa, double c0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    for (int c = 0; c < 3; ++c) soa[(size_t)c * M + k] = c0 * aos[3 * k + c];
}
// aos[3k + c] += c0 * soa[c*M + k]
__global__ void k_soa_add_aos(int M, const double* __restrict__ soa, double* __restrict__ aos, double c0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    for (int c = 0; c < 3; ++c) aos[3 * k + c] += c0 * soa[(size_t)c * M + k];
}
}  // namespace

void launch_aos_to_soa(int M, const double* aos, double* soa, double c0, cudaStream_t s) {
    if (M > 0) k_aos_to_soa<<<(M + 255) / 256, 256, 0, s>>>(M, aos, soa, c0);
}
void launch_soa_add_aos(int M, const double* soa, double* aos, double c0, cudaStream_t s) {
    if (M > 0) k_soa_add_aos<<<(M + 255) / 256, 256, 0, s>>>(M, soa, aos, c0);
}
}  // namespace afmib
