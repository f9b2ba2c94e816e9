// Shared device-side definitions for the afmib GB300 kernels (sm_103a).
//
// Field layout in HBM: every field is one flat array, x fastest,
// i = x + nx*(y + ny*z). Velocity lives on MAC faces: u[i] at (x, y+1/2, z+1/2),
// v[i] at (x+1/2, y, z+1/2), w[i] at (x+1/2, y+1/2, z), in units of h = 1/n.
// In channel mode (walls at y = 0 and y = ny, the reference's domain) v keeps
// all ny planes and plane y = 0 is the bottom wall, held at zero; the top wall
// face y = ny is the periodic image of plane 0. With that convention the
// advection, divergence, gradient and v-Helmholtz stencils of the channel are
// the periodic stencils (every wall term carries a zero factor), and only the
// pressure Laplacian, the multigrid transfers and the u/w Helmholtz wall rows
// need channel-specific code.
#pragma once

#include <cstdlib>

#include <cuda_runtime.h>
#include <stdint.h>

namespace afmib {

struct Dims {
    int nx, ny, nz;  // cells
    int n;           // cells per unit length
    int channel;     // 1: walls in y
    __host__ __device__ long long sxy() const { return (long long)nx * ny; }
    __host__ __device__ long long ncell() const { return (long long)nx * ny * nz; }
};

__host__ __device__ inline int wrapi(int i, int m) {
    i %= m;
    return i < 0 ? i + m : i;
}

__device__ __forceinline__ long long lin(const Dims& d, int x, int y, int z) {
    return (long long)x + (long long)d.nx * ((long long)y + (long long)d.ny * z);
}

// neighbour offsets along each axis with periodic wrap
__device__ __forceinline__ int xm1(const Dims& d, int x) { return x == 0 ? d.nx - 1 : x - 1; }
__device__ __forceinline__ int xp1(const Dims& d, int x) { return x == d.nx - 1 ? 0 : x + 1; }
__device__ __forceinline__ int ym1(const Dims& d, int y) { return y == 0 ? d.ny - 1 : y - 1; }
__device__ __forceinline__ int yp1(const Dims& d, int y) { return y == d.ny - 1 ? 0 : y + 1; }
__device__ __forceinline__ int zm1(const Dims& d, int z) { return z == 0 ? d.nz - 1 : z - 1; }
__device__ __forceinline__ int zp1(const Dims& d, int z) { return z == d.nz - 1 ? 0 : z + 1; }

// Index arithmetic for power-of-two extents with fewer than 2^31 cells: 32-bit
// indices composed by shifts, periodic wraps by masks. On GB300 the generic
// 64-bit index and conditional wraps cost the batched FP32 stencils about a
// third of their time.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ int log2p2(int v) { return __ffs(v) - 1; }
#else
inline int log2p2(int v) { return __builtin_ctz((unsigned)v); }
#endif
struct Ix2 {
    int mx, my, mz, lx, lxy;
    __host__ __device__ __forceinline__ explicit Ix2(const Dims& d)
        : mx(d.nx - 1), my(d.ny - 1), mz(d.nz - 1), lx(log2p2(d.nx)), lxy(log2p2(d.nx) + log2p2(d.ny)) {}
    __device__ __forceinline__ int at(int x, int y, int z) const { return x | (y << lx) | (z << lxy); }
    __device__ __forceinline__ int xm(int x) const { return (x - 1) & mx; }
    __device__ __forceinline__ int xp(int x) const { return (x + 1) & mx; }
    __device__ __forceinline__ int ym(int y) const { return (y - 1) & my; }
    __device__ __forceinline__ int yp(int y) const { return (y + 1) & my; }
    __device__ __forceinline__ int zm(int z) const { return (z - 1) & mz; }
    __device__ __forceinline__ int zp(int z) const { return (z + 1) & mz; }
};
// Block coordinates, walked from the grid's far end when rev. Blocks are
// dispatched roughly in index order, so a pass over a field larger than L2
// that runs opposite to the pass before it starts on the rows that pass
// left in L2 (results are unchanged: the kernels that take it are pointwise
// or update one red-black colour).
__device__ __forceinline__ uint3 block_at(int rev) {
    return rev ? make_uint3(gridDim.x - 1 - blockIdx.x, gridDim.y - 1 - blockIdx.y, gridDim.z - 1 - blockIdx.z)
               : blockIdx;
}

// Power-of-two kernels apply; AFMIB_IX2=0 keeps the general kernels (read at
// every launch, so a test can compare both in one process).
inline bool ix2_ok(const Dims& d) {
    auto p2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
    if (const char* e = std::getenv("AFMIB_IX2"))
        if (e[0] == '0') return false;
    return p2(d.nx) && p2(d.ny) && p2(d.nz) && d.ncell() < (1ll << 31);
}

// ---------------------------------------------------------------------------
// Deterministic grid-wide sums. Each block reduces its values with warp
// shuffles in a fixed tree, writes one partial, and the last block to finish
// (atomic ticket) sums the partials in a fixed order. The result therefore
// does not depend on block scheduling. `scratch` holds the partials and the
// ticket; the ticket is left at zero for the next launch.
// ---------------------------------------------------------------------------
constexpr int kRedBlock = 256;
constexpr int kMaxRedBlocks = 8192;

struct RedScratch {
    double* partial;     // [kMaxRedBlocks * kMaxRedVals]
    unsigned* ticket;    // [1]
};
constexpr int kMaxRedVals = 4;

template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// linear thread / block indices for 1-D, 2-D and 3-D launches
__device__ __forceinline__ int tid_lin() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ __forceinline__ int bid_lin() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ __forceinline__ int nblk_lin() { return gridDim.x * gridDim.y * gridDim.z; }

// Block-wide sum of NV values (TB threads per block); result valid in thread 0.
template <int NV, int TB = kRedBlock>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double s[TB / 32][NV];
    warp_sum<NV>(v);
    const int w = tid_lin() >> 5, l = tid_lin() & 31;
    if (l == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) s[w][k] = v[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = (l < TB / 32) ? s[l][k] : 0.0;
        warp_sum<NV>(v);
    }
    __syncthreads();
}

// Reduce v over the whole grid into out[0..NV-1]. Must be reached by every
// thread of every block exactly once. Returns true in exactly one thread (the
// finisher: thread 0 of the last block), where v then holds the totals, so
// that a caller can derive further scalars (CG coefficients) in place.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], RedScratch sc, double* out) {
    __shared__ bool last;
    block_sum<NV>(v);
    const int tid = tid_lin(), nb = nblk_lin();
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) sc.partial[(size_t)k * kMaxRedBlocks + bid_lin()] = v[k];
        __threadfence();
        unsigned t = atomicAdd(sc.ticket, 1u);
        last = (t == (unsigned)nb - 1);
    }
    __syncthreads();
    if (last) {
        __threadfence();
        double a[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) a[k] = 0.0;
        for (int b = tid; b < nb; b += kRedBlock)
#pragma unroll
            for (int k = 0; k < NV; ++k) a[k] += __ldcg(&sc.partial[(size_t)k * kMaxRedBlocks + b]);
        block_sum<NV>(a);
        if (tid == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                out[k] = a[k];
                v[k] = a[k];
            }
            *sc.ticket = 0u;
            return true;
        }
    }
    return false;
}

// Stencil reductions run on (32 x 8)-thread blocks over (x, y) tiles with
// each thread walking z in steps of grid.z, so that no linear index is ever
// divided; grid.z is chosen for about kRedWaveBlocks blocks, at most
// kMaxRedBlocks.
constexpr int kRBX = 32, kRBY = 8;
// Blocks per grid: about four full waves of the 152 SMs at eight resident
// 256-thread blocks each, so that the last wave is not a fraction.
constexpr int kRedWaveBlocks = 152 * 8 * 4;
inline dim3 red_grid3(int nx, int ny, int nz) {
    const int gx = (nx + kRBX - 1) / kRBX, gy = (ny + kRBY - 1) / kRBY;
    int gz = (kRedWaveBlocks + gx * gy - 1) / (gx * gy);
    if (gz * gx * gy > kMaxRedBlocks) gz = kMaxRedBlocks / (gx * gy);
    if (gz > nz) gz = nz;
    if (gz < 1) gz = 1;
    return dim3(gx, gy, gz);
}

// Persistent form of the same walk, for a stencil reduction that runs beside
// kernels on another stream: a 1-D grid of a few blocks per SM (so that the
// other stream's blocks find free SM slots) strides over (tile, z) items in
// z-major order. The cells each thread visits and their values are those of
// the red_grid3 form; only the order of the reduction's partial sums differs.
inline dim3 walk_grid(const Dims& d, int blocks) {
    const long long items =
        (long long)((d.nx + kRBX - 1) / kRBX) * ((d.ny + kRBY - 1) / kRBY) * d.nz;
    long long b = blocks;
    if (b > items) b = items;
    if (b > kMaxRedBlocks) b = kMaxRedBlocks;
    if (b < 1) b = 1;
    return dim3((unsigned)b);
}
template <typename F>
__device__ __forceinline__ void tile_walk(const Dims& d, F&& body) {
    const int gx = (d.nx + kRBX - 1) / kRBX, gxy = gx * ((d.ny + kRBY - 1) / kRBY);
    const long long items = (long long)gxy * d.nz;
#pragma unroll 2
    for (long long it = blockIdx.x; it < items; it += gridDim.x) {
        const int t = (int)(it % gxy), zi = (int)(it / gxy);
        const int xi = (t % gx) * kRBX + threadIdx.x, yi = (t / gx) * kRBY + threadIdx.y;
        if (xi < d.nx && yi < d.ny) body(xi, yi, zi);
    }
}

// First FP64 defects of the mixed form: the double-float pair by integer
// operations (AFMIB_LO_SPLIT=0: hardware rounding and an FP64 difference)
inline bool lo_split() {
    const char* e = std::getenv("AFMIB_LO_SPLIT");
    return !(e && e[0] == '0');
}

// Resident blocks per SM the double-float residual updates are compiled for
// (registers capped at 40, a few bytes spilled): more loads in flight; at
// 256^3 50.2 IB steps/s against 48.5 uncapped (66 registers) and 48.6 for 8
// blocks (32 registers, heavy spills).
constexpr int kUpdateMinBlocks = 6;

// Per-thread partial sums stay in the arithmetic type (one FP64 conversion
// per thread, not per element: on GB300 conversions run on the FP64 pipe).
template <typename T>
struct Acc {
    T v = T(0);
    __device__ void add(T x) { v += x; }
};

inline int red_blocks(long long n) {
    long long b = (n + kRedBlock - 1) / kRedBlock;
    if (b > kRedWaveBlocks) b = kRedWaveBlocks;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace afmib
