// Immersed-boundary transfer kernels: springs, marker binning by a stable
// device radix sort, deterministic gather spreading and interpolation.
//
// Reference: ib::grid::interpolate (src/ib/grid.h:68-84) computes both
// directions face by face or marker by marker with the cosine 4-point kernel
//   phi(r) = n/4 (1 + cos(pi r n / 2)), |r n| <= 2     (src/ib/grid.h:51-55)
// and finds neighbours with a kd-tree (src/dt/kdtree.h). Here the markers are
// binned by cell instead: a key (tile, cell in tile) per marker is sorted with
// a stable LSD radix sort, so the markers of every cell are contiguous and in
// index order. Spreading then runs one block per output tile of TS^3 cells,
// gathering from the markers binned in the tile's (TS+4)^3 neighbourhood in a
// fixed order: no float atomics, bitwise repeatable.
//
// Weights: for a marker at s = X*n along an axis and faces at j + off, the
// four faces with |j + off - s| < 2 are j = floor(s - off) - 1 + m, m = 0..3,
// and with t = frac(s - off), S = sin(pi t / 2), C = cos(pi t / 2):
//   phi/n = (1 - S)/4, (1 + C)/4, (1 + S)/4, (1 - C)/4      (sum = 1)
// (cos(pi r/2) at r = -1-t, -t, 1-t, 2-t). One sincospi per axis and offset.
#include <type_traits>

#include "dfloat.cuh"
#include "kernels_ib.h"

namespace afmib {

namespace {

__device__ __forceinline__ double sinpi_cospi(double x, double* c) {
    double s;
    sincospi(x, &s, c);
    return s;
}
__device__ __forceinline__ float sinpi_cospi(float x, float* c) {
    float s;
    sincospif(x, &s, c);
    return s;
}

// G_i = k * sum_j (X_j - X_i)
template <typename T>
__global__ void k_springs(int M, const double* __restrict__ X, const int* __restrict__ ns, const int* __restrict__ ni,
                          double k, T* __restrict__ G) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2];
    double sx = 0, sy = 0, sz = 0;
    for (int e = ns[i]; e < ns[i + 1]; ++e) {
        const int j = ni[e];
        sx += X[3 * j] - xi;
        sy += X[3 * j + 1] - yi;
        sz += X[3 * j + 2] - zi;
    }
    G[i] = T(k * sx);
    G[M + i] = T(k * sy);
    G[2 * M + i] = T(k * sz);
}

// Y = L X per marker (L the graph Laplacian of the spring lists), stored
// like X: Y_i = sum_{j in N(i)} (X_j - X_i)
__global__ void k_lap_aos(int M, const double* __restrict__ X, const int* __restrict__ ns, const int* __restrict__ ni,
                          double* __restrict__ Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2];
    double sx = 0, sy = 0, sz = 0;
    for (int e = ns[i]; e < ns[i + 1]; ++e) {
        const int j = ni[e];
        sx += X[3 * j] - xi;
        sy += X[3 * j + 1] - yi;
        sz += X[3 * j + 2] - zi;
    }
    Y[3 * i] = sx;
    Y[3 * i + 1] = sy;
    Y[3 * i + 2] = sz;
}

// Springs plus bending from Y = L X: G_i = ks Y_i - kb (L Y)_i. The bending
// term is the force of the discrete energy kb/2 sum_i |(L X)_i|^2 (with
// symmetric lists L is symmetric, so the gradient is kb L L X).
template <typename T>
__global__ void k_spring_bend(int M, const double* __restrict__ Y, const int* __restrict__ ns,
                              const int* __restrict__ ni, double ks, double kb, T* __restrict__ G) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const double yi[3] = {Y[3 * i], Y[3 * i + 1], Y[3 * i + 2]};
    double b[3] = {0, 0, 0};
    for (int e = ns[i]; e < ns[i + 1]; ++e) {
        const int j = ni[e];
        for (int a = 0; a < 3; ++a) b[a] += Y[3 * j + a] - yi[a];
    }
    for (int a = 0; a < 3; ++a) G[(size_t)a * M + i] = T(ks * yi[a] - kb * b[a]);
}

// Per marker: bin key, wrapped cell, and for each axis and offset variant
// (0: faces on integer positions, 1: on half-integers) the base offset
// (first face - cell) and the four weights phi/n.
// DF (FP64 weights only): the sine and cosine by df_sincospi on the FP32
// pipe instead of the FP64 sincospi (the mixed form), weights rounded to FP64
// from their pairs
template <typename T, bool DF>
__global__ void k_marker_prep(Dims d, int TS, int M, const double* __restrict__ X, unsigned* __restrict__ keys,
                              int* __restrict__ vals, MarkerW<T> mw, int* __restrict__ flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    const int ext[3] = {d.nx, d.ny, d.nz};
    const int TZ = d.nz == 1 ? 1 : TS;  // 2D grids: tiles one cell deep
    int cell[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double s = X[3 * k + a] * d.n;
        const double fs = floor(s);
        cell[a] = wrapi((int)fs, ext[a]);
        if (a == 1 && d.channel && (s < 2.5 || s > d.ny - 2.5)) atomicExch(flag, 1);
        if (!(s == s)) atomicExch(flag, 2);
        if (a == 2 && d.nz == 1) {
            // 2D: the z kernel is the single plane with weight one
            cell[2] = 0;
#pragma unroll
            for (int v = 0; v < 2; ++v) {
                mw.dbase[(k * 3 + a) * 2 + v] = 0;
                T* w = mw.w + (((size_t)k * 3 + a) * 2 + v) * 4;
                w[0] = T(1);
                w[1] = w[2] = w[3] = T(0);
            }
            continue;
        }
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const double t = s - 0.5 * v;
            const double ft = floor(t);
            const T frac = T(t - ft);
            mw.dbase[(k * 3 + a) * 2 + v] = (signed char)((int)ft - 1 - (int)fs);
            T* w = mw.w + (((size_t)k * 3 + a) * 2 + v) * 4;
            if constexpr (DF && sizeof(T) == sizeof(double)) {
                df2 hx = df_split(frac);  // frac / 2 exactly
                hx.hi *= 0.5f;
                hx.lo *= 0.5f;
                df2 Sx, Cx;
                df_sincospi(hx, &Sx, &Cx);
                const df2 one = {1.f, 0.f};
                const df2 q[4] = {df_add(one, df_neg(Sx)), df_add(one, Cx), df_add(one, Sx), df_add(one, df_neg(Cx))};
#pragma unroll
                for (int m = 0; m < 4; ++m) w[m] = f32_to_f64(0.25f * q[m].hi) + f32_to_f64(0.25f * q[m].lo);
            } else {
                T C;
                const T S = sinpi_cospi(frac * T(0.5), &C);
                w[0] = T(0.25) * (T(1) - S);
                w[1] = T(0.25) * (T(1) + C);
                w[2] = T(0.25) * (T(1) + S);
                w[3] = T(0.25) * (T(1) - C);
            }
        }
    }
    mw.cell[3 * k] = cell[0];
    mw.cell[3 * k + 1] = cell[1];
    mw.cell[3 * k + 2] = cell[2];
    const int tx = cell[0] / TS, ty = cell[1] / TS, tz = cell[2] / TZ;
    const int ntx = d.nx / TS, nty = d.ny / TS;
    const unsigned tile = (unsigned)(tx + ntx * (ty + nty * tz));
    const unsigned local = (unsigned)((cell[0] % TS) + TS * ((cell[1] % TS) + TS * (cell[2] % TZ)));
    if (keys) keys[k] = tile * (unsigned)(TS * TS * TZ) + local;  // null: weights only
    if (vals) vals[k] = k;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (key, value) pairs, 8-bit digits.
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned* __restrict__ keys, int n, int shift,
                                                        unsigned* __restrict__ hist, int nblk) {
    __shared__ unsigned cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan of hist[256 * nblk] in one block of 1024 threads
__global__ void __launch_bounds__(1024) k_rs_scan(unsigned* __restrict__ hist, int total) {
    __shared__ unsigned part[1024];
    const int per = (total + 1023) / 1024;
    const int lo = threadIdx.x * per, hi = min(lo + per, total);
    unsigned s = 0;
    for (int i = lo; i < hi; ++i) s += hist[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        unsigned v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = part[threadIdx.x] - s;
    for (int i = lo; i < hi; ++i) {
        const unsigned c = hist[i];
        hist[i] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned* __restrict__ kin, const int* __restrict__ vin,
                                                           unsigned* __restrict__ kout, int* __restrict__ vout, int n,
                                                           int shift, const unsigned* __restrict__ hist, int nblk) {
    __shared__ unsigned s_off[256];
    __shared__ unsigned s_wcnt[RS_THREADS / 32][256];
    __shared__ unsigned s_wpre[RS_THREADS / 32][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    s_off[threadIdx.x] = hist[threadIdx.x * nblk + blockIdx.x];
    for (int w = 0; w < RS_THREADS / 32; ++w) s_wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int i = base + r * RS_THREADS + threadIdx.x;
        const bool valid = i < n;
        const unsigned key = valid ? kin[i] : 0u;
        const int val = valid ? vin[i] : 0;
        const unsigned dig = valid ? ((key >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, dig);
        const unsigned rank = __popc(peers & lt);
        if (valid && lane == __ffs(peers) - 1) s_wcnt[warp][dig] = __popc(peers);
        __syncthreads();
        {
            unsigned run = s_off[threadIdx.x];
            for (int w = 0; w < RS_THREADS / 32; ++w) {
                const unsigned c = s_wcnt[w][threadIdx.x];
                s_wpre[w][threadIdx.x] = run;
                run += c;
                s_wcnt[w][threadIdx.x] = 0;
            }
            s_off[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            const unsigned pos = s_wpre[warp][dig] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

// tile ranges of the sorted keys: tstart/tend zeroed beforehand
__global__ void k_tile_ranges(const unsigned* __restrict__ keys, int M, int cells_per_tile, int* __restrict__ tstart,
                              int* __restrict__ tend) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    const unsigned t = keys[p] / (unsigned)cells_per_tile;
    if (p == 0 || keys[p - 1] / (unsigned)cells_per_tile != t) tstart[t] = p;
    if (p == M - 1 || keys[p + 1] / (unsigned)cells_per_tile != t) tend[t] = p + 1;
}

// Per tile: slot of each occupied tile (or -1) and the list of output tiles
// whose (TS+4)^3 neighbourhood holds a marker. Slots are handed out by an
// atomic counter; a slot only names storage, so its value never reaches a result.
__global__ void k_active_tiles(int ntx, int nty, int ntz, int channel, const int* __restrict__ tstart,
                               const int* __restrict__ tend, int* __restrict__ list, int* __restrict__ count,
                               int* __restrict__ slot, int* __restrict__ occ, int* __restrict__ occ_count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntx * nty * ntz) return;
    if (tend[t] > tstart[t]) {
        const int sl = atomicAdd(occ_count, 1);
        slot[t] = sl;
        occ[sl] = t;
    } else {
        slot[t] = -1;
    }
    const int tx = t % ntx, ty = (t / ntx) % nty, tz = t / (ntx * nty);
    bool any = false;
    for (int dz = -1; dz <= 1 && !any; ++dz)
        for (int dy = -1; dy <= 1 && !any; ++dy) {
            int yy = ty + dy;
            if (channel && (yy < 0 || yy >= nty)) continue;
            yy = wrapi(yy, nty);
            for (int dx = -1; dx <= 1 && !any; ++dx) {
                const int n = wrapi(tx + dx, ntx) + ntx * (yy + nty * wrapi(tz + dz, ntz));
                if (tend[n] > tstart[n]) any = true;
            }
        }
    if (any) list[atomicAdd(count, 1)] = t;
}

// Cell-start table of every occupied tile: ctab[slot][c] = first sorted
// position of local cell c (c = TS^3 holds the tile's end), by binary search
// in the tile's sorted key range.
template <int TS, int TZ>
__global__ void __launch_bounds__(TS * TS * TZ) k_cell_table(const unsigned* __restrict__ keys,
                                                            const int* __restrict__ tstart, const int* __restrict__ tend,
                                                            const int* __restrict__ occ, const int* __restrict__ occ_count,
                                                            int* __restrict__ ctab) {
    constexpr int C = TS * TS * TZ;
    const int nocc = *occ_count;
    for (int li = blockIdx.x; li < nocc; li += gridDim.x) {
        const int t = occ[li];
        const int a = tstart[t], b = tend[t];
        const unsigned key = (unsigned)t * C + threadIdx.x;
        int lo = a, hi = b;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (keys[mid] < key) lo = mid + 1; else hi = mid;
        }
        int* row = ctab + (size_t)li * (C + 1);
        row[threadIdx.x] = lo;
        if (threadIdx.x == 0) row[C] = b;
    }
}

// Compute types of the gather: T itself (FP64, FP32) or, for FP64 inputs in
// the mixed form, dfl: the weight products and the face sums carried as
// double-float pairs (relative 2^-44) on the FP32 pipe, GB300's FP64 pipe
// being 1/64 of it. Inputs are split exactly by integer operations
// (df_split), the sum goes back to FP64 with one addition per face.
struct dfl {
    df2 v;
};
__device__ __forceinline__ dfl operator*(dfl a, dfl b) { return dfl{df_mul(a.v, b.v)}; }
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) {
    a.v = df_add(a.v, b.v);
    return a;
}
template <typename TC>
__device__ __forceinline__ TC tc_from(double v) { return TC(v); }
template <>
__device__ __forceinline__ dfl tc_from<dfl>(double v) { return dfl{df_split(v)}; }
template <typename T, typename TC>
__device__ __forceinline__ T tc_to(TC v) { return T(v); }
template <>
__device__ __forceinline__ double tc_to<double, dfl>(dfl v) { return f32_to_f64(v.v.hi) + f32_to_f64(v.v.lo); }

// ---------------------------------------------------------------------------
// Gather spreading. One block (TS^3 threads, one face per component each) per
// active output tile. The markers binned in E = the tile grown by two cells
// per side are staged in shared memory in E-cell order (x fastest): every E
// row (ey, ez) is cut into at most three tile segments, each a contiguous run
// of the sorted markers, and one block scan of the segment lengths places the
// runs. A face at E-local J gathers cells [J-2, J+1] along its own axis and
// [J-2, J+2] along the other two, i.e. at most 25 contiguous runs, in a fixed
// order: no float atomics, bitwise repeatable.
// A tile whose neighbourhood holds more than `cap` markers is either left to
// a second, larger-capacity launch (ovf_list given) or, in that launch,
// spread in chunks of `cap` staged markers. A face visits its runs in
// increasing staged order (rows ascend in E-linear order), so cutting that
// order into chunks leaves every face's summation order, and its result bits,
// unchanged: there is no marker-density limit.
// ---------------------------------------------------------------------------
template <typename T, int TS, int TZ, typename TC = T>
__global__ void __launch_bounds__(TS * TS * TZ) k_spread_gather(Dims d, int M, const int* __restrict__ perm,
                                                                MarkerW<T> mw, const T* __restrict__ G,
                                                                const double* __restrict__ vol, double scale,
                                                                const int* __restrict__ slot, const int* __restrict__ ctab,
                                                                const int* __restrict__ list, const int* __restrict__ count,
                                                                int cap, T* __restrict__ fu, T* __restrict__ fv,
                                                                T* __restrict__ fw,
                                                                int* __restrict__ ovf_list, int* __restrict__ ovf_count,
                                                                int* __restrict__ next_tile) {
    // 3D: TZ == TS, the neighbourhood grows by 2 cells per side along every
    // axis. 2D (TZ == 1, nz == 1): one plane, no z halo.
    constexpr int NT = TS * TS * TZ, E = TS + 4, EZ = TZ == 1 ? 1 : TS + 4, HZ = TZ == 1 ? 0 : 2;
    constexpr int E2 = E * E, E3 = E2 * EZ, C = TS * TS * TZ;
    constexpr int CPT = (E3 + NT - 1) / NT;  // consecutive E cells per thread
    extern __shared__ __align__(16) unsigned char smem[];
    int* s_estart = (int*)smem;          // E3 + 1: first staged slot of each E cell
    int* s_scan = s_estart + (E3 + 1);   // NT / 32: warp totals of the block scan
    int* s_k = s_scan + NT;              // cap: marker index of each staged slot
    int* s_base = s_k + cap;             // cap: packed E-local first faces
    // cap * 12: x weights, y weights, z weights times the marker's force
    TC* s_w = (TC*)(((uintptr_t)(s_base + cap) + 15) & ~(uintptr_t)15);

    const int ntx = d.nx / TS, nty = d.ny / TS;
    const int ncount = *count;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int lx = tid % TS, ly = (tid / TS) % TS, lz = tid / (TS * TS);
    auto wrap1 = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };
    // tiles are taken from a shared counter (their costs differ widely near a
    // membrane); each tile is still computed by one block, in a fixed order
    __shared__ int s_li;
    for (;;) {
        __syncthreads();
        if (tid == 0) s_li = atomicAdd(next_tile, 1);
        __syncthreads();
        const int li = s_li;
        if (li >= ncount) break;
        const int t = list[li];
        const int tx = t % ntx, ty = (t / ntx) % nty, tz = t / (ntx * nty);
        const int ox = tx * TS - 2, oy = ty * TS - 2, oz = tz * TZ - HZ;  // E origin (unwrapped cells)
        // sorted run [p0, p0 + cnt) of the markers binned in E cell e
        auto run_of = [&](int e, int& p0, int& cnt) {
            p0 = 0;
            cnt = 0;
            const int ex = e % E, ey = (e / E) % E, ez = e / E2;
            const int gy = oy + ey;
            if (d.channel && (gy < 0 || gy >= d.ny)) return;
            const int gx = wrap1(ox + ex, d.nx), gyw = wrap1(gy, d.ny), gz = wrap1(oz + ez, d.nz);
            const int sl = slot[gx / TS + ntx * (gyw / TS + nty * (gz / TZ))];
            if (sl < 0) return;
            const int lc = (gx % TS) + TS * ((gyw % TS) + TS * (gz % TZ));
            const int* row = ctab + (size_t)sl * (C + 1) + lc;
            p0 = row[0];
            cnt = row[1] - p0;
        };
        // ---- markers of each E cell (E-linear order e = ex + E (ey + E ez)):
        //      thread tid takes cells [tid * CPT, tid * CPT + CPT), whose
        //      cell-table loads are independent of one another
        int cnt[CPT], p0[CPT];
        int tot = 0;
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            const int e = tid * CPT + k;
            cnt[k] = 0;
            p0[k] = 0;
            if (e < E3) run_of(e, p0[k], cnt[k]);
            tot += cnt[k];
        }
        // ---- block exclusive scan of the per-thread totals (thread order = E order);
        //      NT < 32 (4 x 4 x 1 tiles) is one partial warp
        constexpr int NW = (NT + 31) / 32;
        constexpr unsigned WMASK = NT >= 32 ? 0xffffffffu : ((1u << NT) - 1u);
        constexpr int WLAST = NT >= 32 ? 31 : NT - 1;
        int inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(WMASK, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == WLAST) s_scan[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            int w = lane < NW ? s_scan[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(WMASK, w, o);
                if (lane >= o) w += v;
            }
            if (lane < NW) s_scan[lane] = w;  // inclusive warp prefix
        }
        __syncthreads();
        const int nc_all = s_scan[NW - 1];
        int off = inc - tot + (warp > 0 ? s_scan[warp - 1] : 0);
        // an active tile whose neighbourhood holds no marker (its occupied
        // neighbour tiles' markers lie beyond the 2-cell halo) adds nothing:
        // its faces keep the zeros the callers wrote (block-uniform)
        if (nc_all == 0) continue;
        const bool chunked = nc_all > cap;  // block-uniform
        if (chunked && ovf_list) {           // left to the large-capacity pass
            if (tid == 0) ovf_list[atomicAdd(ovf_count, 1)] = t;
            continue;
        }
        // ---- E-cell starts and, in one pass, the staged marker indices
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            const int e = tid * CPT + k;
            if (e < E3) {
                s_estart[e] = off;
                if (!chunked)
                    for (int m = 0; m < cnt[k]; ++m) s_k[off + m] = perm[p0[k] + m];
                off += cnt[k];
            }
        }
        if (tid == 0) s_estart[E3] = nc_all;
        const int nchunk = chunked ? (nc_all + cap - 1) / cap : 1;
        // chunked: marker indices of staged slots [lo, lo + cap) from this
        // thread's E cells (runs looked up again: nothing held across chunks)
        auto stage_ids = [&](int lo) {
            for (int k = 0; k < CPT; ++k) {
                const int e = tid * CPT + k;
                if (e >= E3) break;
                const int o = s_estart[e], n = s_estart[e + 1] - o;
                if (n == 0 || o + n <= lo || o >= lo + cap) continue;
                int q0, qn;
                run_of(e, q0, qn);
                const int a = lo - o > 0 ? lo - o : 0, b = lo + cap - o < n ? lo + cap - o : n;
                for (int m = a; m < b; ++m) s_k[o + m - lo] = perm[q0 + m];
            }
        };
        __syncthreads();
        // ---- one component at a time (and, past the capacity, one chunk at a time)
        const int J[3] = {lx + 2, ly + 2, lz + HZ};
        for (int comp = 0; comp < 3; ++comp) {
            TC acc = tc_from<TC>(0.0);
            const unsigned jp = 0x00808080u | (unsigned)(J[0] + 8) | ((unsigned)(J[1] + 8) << 8) |
                                ((unsigned)(J[2] + 8) << 16);
            const int hx = (comp == 0) ? J[0] + 1 : J[0] + 2;
            const int hy = (comp == 1) ? J[1] + 1 : J[1] + 2;
            const int hz = TZ == 1 ? J[2] : ((comp == 2) ? J[2] + 1 : J[2] + 2);
            for (int ch = 0; ch < nchunk; ++ch) {
                const int lo = ch * cap, nc = nc_all - lo < cap ? nc_all - lo : cap;
                if (chunked) {
                    __syncthreads();  // the previous chunk's gather is done with s_k, s_base, s_w
                    stage_ids(lo);
                    __syncthreads();
                }
                for (int sl = tid; sl < nc; sl += NT) {
                    const int k = s_k[sl];
                    const TC g = tc_from<TC>((double)G[(size_t)comp * M + k] * (vol ? vol[k] : 1.0) * scale);
                    int packed = 0;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const int v = (a == comp) ? 0 : 1;
                        const int o = a == 0 ? ox : (a == 1 ? oy : oz);
                        const int n_a = a == 0 ? d.nx : (a == 1 ? d.ny : d.nz);
                        // E-local first face: cell relative to the E origin + offset
                        int ec = mw.cell[3 * k + a] - o;
                        if (!(a == 1 && d.channel)) ec = wrapi(ec, n_a);
                        const int b = ec + mw.dbase[(k * 3 + a) * 2 + v];
                        packed |= (b + 8) << (8 * a);
                        const T* w = mw.w + (((size_t)k * 3 + a) * 2 + v) * 4;
#pragma unroll
                        for (int m = 0; m < 4; ++m)
                            s_w[(size_t)sl * 12 + a * 4 + m] = a == 2 ? tc_from<TC>(w[m]) * g : tc_from<TC>(w[m]);
                    }
                    s_base[sl] = packed;
                }
                __syncthreads();
                for (int ez = J[2] - HZ; ez <= hz; ++ez)
                    for (int ey = J[1] - 2; ey <= hy; ++ey) {
                        const int row = E * (ey + E * ez);
                        int s0 = s_estart[row + J[0] - 2] - lo, s1 = s_estart[row + hx + 1] - lo;
                        s0 = s0 > 0 ? s0 : 0;
                        s1 = s1 < nc ? s1 : nc;
                        for (int sl = s0; sl < s1; ++sl) {
                            // per byte (0x80 + J + 8) - (b + 8): no borrow crosses a
                            // byte (all fields < 0x80); the face is in the marker's
                            // support iff every byte is 0x80 + {0..3}
                            const unsigned t = jp - (unsigned)s_base[sl];
                            if ((t & 0x00FCFCFCu) == 0x00808080u) {
                                const TC* w = s_w + (size_t)sl * 12;
                                acc += (w[t & 3u] * w[4 + ((t >> 8) & 3u)]) * w[8 + ((t >> 16) & 3u)];
                            }
                        }
                    }
            }
            T* f = comp == 0 ? fu : (comp == 1 ? fv : fw);
            const int gx = tx * TS + lx, gy = ty * TS + ly, gz = tz * TZ + lz;
            if (!(d.channel && comp == 1 && gy == 0)) f[lin(d, gx, gy, gz)] = tc_to<T, TC>(acc);
            __syncthreads();
        }
    }
}

// Interpolation U_k = sum over 4^3 faces of (phi/n)^3 * u(face)
// (src/ib/grid.h:68-84 with volume h^3, src/ib/eulerian_grid.h:45).
template <typename T, typename TF>
__global__ void k_interp(Dims d, int M, const int* __restrict__ perm, MarkerW<T> mw, const TF* __restrict__ u,
                         const TF* __restrict__ v, const TF* __restrict__ w, double* __restrict__ U) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    const int k = perm ? perm[p] : p;
    const int ext[3] = {d.nx, d.ny, d.nz};
    for (int comp = 0; comp < 3; ++comp) {
        const TF* src = comp == 0 ? u : (comp == 1 ? v : w);
        int idx[3][4];
        T wt[3][4];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int var = (a == comp) ? 0 : 1;
            const int b = mw.cell[3 * k + a] + mw.dbase[(k * 3 + a) * 2 + var];
            const T* ww = mw.w + (((size_t)k * 3 + a) * 2 + var) * 4;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                idx[a][m] = wrapi(b + m, ext[a]);
                wt[a][m] = ww[m];
            }
        }
        T acc = T(0);
#pragma unroll
        for (int mz = 0; mz < 4; ++mz)
#pragma unroll
            for (int my = 0; my < 4; ++my) {
                const T wyz = wt[1][my] * wt[2][mz];
                const long long row = (long long)d.nx * (idx[1][my] + (long long)d.ny * idx[2][mz]);
#pragma unroll
                for (int mx = 0; mx < 4; ++mx) acc += wt[0][mx] * wyz * T(src[row + idx[0][mx]]);
            }
        U[(size_t)comp * M + k] = (double)acc;
    }
}

// The same interpolation of FP64 fields in double-float on the FP32 pipe
// (the mixed form; GB300's FP64 pipe runs at 1/64 of the FP32 rate). Four
// lanes take one marker, one x tap each: a lane issues the loads of its 16
// (y, z) faces of a component back to back (the fields are larger than L2,
// so the time is DRAM latency), sums them as sum_z wz sum_y wy u, takes its
// x weight, and the quad adds its four partial sums by shuffles in a fixed
// pattern (the first lane's result is stored). Field values and weights are
// split exactly by integer operations (df_split, 24 + 23 bits); each product
// is a pair (fma two-product plus the cross terms) and the sums keep an
// exact two-sum of the leading words and a plain sum of the trailing ones, so
// the result is within a few units of 2^-46 of the largest term times the 4
// to 16 terms of a sum. One FP64 addition per component turns the pair back
// into FP64.
struct DfAcc {
    float s, e;  // leading sum (two-summed), trailing sum
};
__device__ __forceinline__ void dfacc_add(DfAcc& a, float p, float pe) {
    const float s = a.s + p;
    const float v = s - a.s;
    a.e += ((a.s - (s - v)) + (p - v)) + pe;
    a.s = s;
}
__device__ __forceinline__ void dfacc_mul_add(DfAcc& a, df2 x, df2 y) {
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    dfacc_add(a, p, e);
}
__device__ __forceinline__ df2 dfacc_pair(DfAcc a) {
    df2 r;
    r.hi = a.s + a.e;
    r.lo = a.e - (r.hi - a.s);
    return r;
}

constexpr int kInterpDfBlock = 128;

template <bool PAIRS>
__global__ void __launch_bounds__(kInterpDfBlock) k_interp_dfl(Dims d, int M, const int* __restrict__ perm,
                                                               MarkerW<double> mw, const double* __restrict__ u,
                                                               const double* __restrict__ v,
                                                               const double* __restrict__ w, const float* __restrict__ uh,
                                                               const float* __restrict__ ul,
                                                               const float* __restrict__ vh,
                                                               const float* __restrict__ vl,
                                                               const float* __restrict__ wh,
                                                               const float* __restrict__ wl, double* __restrict__ U) {
    const int p = (blockIdx.x * kInterpDfBlock + threadIdx.x) >> 2;
    const int q = threadIdx.x & 3;
    if (p >= M) return;  // a quad leaves together
    const unsigned qmask = 0xfu << (threadIdx.x & 28);
    const int k = perm ? perm[p] : p;
#pragma unroll 1
    for (int comp = 0; comp < 3; ++comp) {
        const double* src = comp == 0 ? u : (comp == 1 ? v : w);
        const int vx = comp == 0 ? 0 : 1, vy = comp == 1 ? 0 : 1, vz = comp == 2 ? 0 : 1;
        const int bx = mw.cell[3 * k] + mw.dbase[(k * 3 + 0) * 2 + vx];
        const int by = mw.cell[3 * k + 1] + mw.dbase[(k * 3 + 1) * 2 + vy];
        const int bz = mw.cell[3 * k + 2] + mw.dbase[(k * 3 + 2) * 2 + vz];
        const long long ix = wrapi(bx + q, d.nx);
        long long roff[4][4];
#pragma unroll
        for (int mz = 0; mz < 4; ++mz)
#pragma unroll
            for (int my = 0; my < 4; ++my)
                roff[mz][my] = (long long)d.nx * (wrapi(by + my, d.ny) + (long long)d.ny * wrapi(bz + mz, d.nz)) + ix;
        df2 val[4][4];
        if (PAIRS) {  // the velocity's float pairs (hi + lo), no splits
            const float* sh = comp == 0 ? uh : (comp == 1 ? vh : wh);
            const float* sl = comp == 0 ? ul : (comp == 1 ? vl : wl);
#pragma unroll
            for (int mz = 0; mz < 4; ++mz)
#pragma unroll
                for (int my = 0; my < 4; ++my) {
                    val[mz][my].hi = sh[roff[mz][my]];
                    val[mz][my].lo = sl[roff[mz][my]];
                }
        } else {
            double dv[4][4];
#pragma unroll
            for (int mz = 0; mz < 4; ++mz)
#pragma unroll
                for (int my = 0; my < 4; ++my) dv[mz][my] = src[roff[mz][my]];
#pragma unroll
            for (int mz = 0; mz < 4; ++mz)
#pragma unroll
                for (int my = 0; my < 4; ++my) val[mz][my] = df_split(dv[mz][my]);
        }
        // the quad's lanes split one y and one z weight each and share them
        const df2 wyq = df_split(mw.w[(((size_t)k * 3 + 1) * 2 + vy) * 4 + q]);
        const df2 wzq = df_split(mw.w[(((size_t)k * 3 + 2) * 2 + vz) * 4 + q]);
        const int q0 = threadIdx.x & 28;
        df2 wy[4], wz[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            wy[m].hi = __shfl_sync(qmask, wyq.hi, q0 + m);
            wy[m].lo = __shfl_sync(qmask, wyq.lo, q0 + m);
            wz[m].hi = __shfl_sync(qmask, wzq.hi, q0 + m);
            wz[m].lo = __shfl_sync(qmask, wzq.lo, q0 + m);
        }
        DfAcc az = {0.f, 0.f};
#pragma unroll
        for (int mz = 0; mz < 4; ++mz) {
            DfAcc ay = {0.f, 0.f};
#pragma unroll
            for (int my = 0; my < 4; ++my) dfacc_mul_add(ay, wy[my], val[mz][my]);
            dfacc_mul_add(az, wz[mz], dfacc_pair(ay));
        }
        const df2 wxq = df_split(mw.w[(((size_t)k * 3 + 0) * 2 + vx) * 4 + q]);
        df2 r = df_mul(wxq, dfacc_pair(az));
        df2 o;
        o.hi = __shfl_xor_sync(qmask, r.hi, 1);
        o.lo = __shfl_xor_sync(qmask, r.lo, 1);
        r = df_add(r, o);
        o.hi = __shfl_xor_sync(qmask, r.hi, 2);
        o.lo = __shfl_xor_sync(qmask, r.lo, 2);
        r = df_add(r, o);
        if (q == 0) U[(size_t)comp * M + k] = f32_to_f64(r.hi) + f32_to_f64(r.lo);
    }
}

// X_out = X_in + c * U  (U component-major)
__global__ void k_marker_axpy(int M, double* __restrict__ Xo, const double* __restrict__ Xi, const double* __restrict__ U,
                              double c) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) Xo[3 * k + a] = Xi[3 * k + a] + c * U[(size_t)a * M + k];
}

}  // namespace

template <typename T>
void launch_springs_bending(int M, const double* X, const int* nstart, const int* nidx, double ks, double kb,
                            double* Y, T* G, cudaStream_t s) {
    if (M <= 0) return;
    k_lap_aos<<<(M + 255) / 256, 256, 0, s>>>(M, X, nstart, nidx, Y);
    k_spring_bend<T><<<(M + 255) / 256, 256, 0, s>>>(M, Y, nstart, nidx, ks, kb, G);
}
template <typename T>
void launch_springs(int M, const double* X, const int* nstart, const int* nidx, double k, T* G, cudaStream_t s) {
    if (M > 0) k_springs<T><<<(M + 255) / 256, 256, 0, s>>>(M, X, nstart, nidx, k, G);
}

template <typename T>
void launch_marker_prep(const Dims& d, int TS, int M, const double* X, unsigned* keys, int* vals, MarkerW<T> mw,
                        int* flag, cudaStream_t s, bool df_weights) {
    if (M <= 0) return;
    if (df_weights && sizeof(T) == sizeof(double))
        k_marker_prep<T, true><<<(M + 255) / 256, 256, 0, s>>>(d, TS, M, X, keys, vals, mw, flag);
    else
        k_marker_prep<T, false><<<(M + 255) / 256, 256, 0, s>>>(d, TS, M, X, keys, vals, mw, flag);
}

size_t radix_sort_temp_bytes(int n) {
    const int nblk = (n + RS_TILE - 1) / RS_TILE;
    return (size_t)256 * (nblk > 0 ? nblk : 1) * sizeof(unsigned);
}

void radix_sort_pairs(unsigned* keys, int* vals, unsigned* keys_alt, int* vals_alt, int n, int bits, unsigned* hist,
                      unsigned** keys_out, int** vals_out, cudaStream_t s) {
    const int nblk = (n + RS_TILE - 1) / RS_TILE;
    unsigned* ka = keys;
    unsigned* kb = keys_alt;
    int* va = vals;
    int* vb = vals_alt;
    for (int shift = 0; shift < bits && n > 0; shift += 8) {
        k_rs_hist<<<nblk, RS_THREADS, 0, s>>>(ka, n, shift, hist, nblk);
        k_rs_scan<<<1, 1024, 0, s>>>(hist, 256 * nblk);
        k_rs_scatter<<<nblk, RS_THREADS, 0, s>>>(ka, va, kb, vb, n, shift, hist, nblk);
        unsigned* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
    }
    *keys_out = ka;
    *vals_out = va;
}

void launch_tile_ranges(const unsigned* keys, int M, int cells_per_tile, int* tstart, int* tend, cudaStream_t s) {
    if (M > 0) k_tile_ranges<<<(M + 255) / 256, 256, 0, s>>>(keys, M, cells_per_tile, tstart, tend);
}

void launch_active_tiles(int ntx, int nty, int ntz, int channel, const int* tstart, const int* tend, int* list,
                         int* count, int* slot, int* occ, int* occ_count, cudaStream_t s) {
    const int nt = ntx * nty * ntz;
    k_active_tiles<<<(nt + 255) / 256, 256, 0, s>>>(ntx, nty, ntz, channel, tstart, tend, list, count, slot, occ,
                                                    occ_count);
}

void launch_cell_table(int TS, int TZ, const unsigned* keys, const int* tstart, const int* tend, const int* occ,
                       const int* occ_count, int max_occ, int* ctab, cudaStream_t s) {
    int blocks = max_occ < 152 * 8 ? max_occ : 152 * 8;
    if (blocks < 1) blocks = 1;
    if (TS == 8 && TZ == 8) k_cell_table<8, 8><<<blocks, 512, 0, s>>>(keys, tstart, tend, occ, occ_count, ctab);
    else if (TS == 4 && TZ == 4) k_cell_table<4, 4><<<blocks, 64, 0, s>>>(keys, tstart, tend, occ, occ_count, ctab);
    else if (TS == 8) k_cell_table<8, 1><<<blocks, 64, 0, s>>>(keys, tstart, tend, occ, occ_count, ctab);
    else k_cell_table<4, 1><<<blocks, 16, 0, s>>>(keys, tstart, tend, occ, occ_count, ctab);
}

template <typename T>
size_t spread_smem_bytes(int TS, int TZ, int cap) {
    const int E = TS + 4, EZ = TZ == 1 ? 1 : TS + 4, E3 = E * E * EZ, NT = TS * TS * TZ;
    size_t ints = (size_t)(E3 + 1) + NT + 2 * (size_t)cap;
    size_t bytes = ints * sizeof(int);
    bytes = (bytes + 15) & ~(size_t)15;
    bytes += (size_t)cap * 12 * sizeof(T);
    return bytes;
}

template <typename T, int TS, int TZ, typename TC>
static void spread_launch(const Dims& d, int M, const int* perm, MarkerW<T> mw, const T* G, const double* vol,
                          double scale, const int* slot, const int* ctab, const int* list, const int* count,
                          int max_tiles, int cap, T* fu, T* fv, T* fw, int* ovf_list, int* ovf_count,
                          int* next_tile, cudaStream_t s) {
    static_assert(sizeof(TC) == sizeof(T), "the staged weights take the input type's size");
    const size_t smem = spread_smem_bytes<T>(TS, TZ, cap);
    // opt in to exactly the dynamic shared memory this launch uses (the
    // kernel's static shared memory counts against the same 227 KB)
    static size_t configured = 0;  // the largest capacity asked for so far
    if (configured < smem) {
        if (cudaFuncSetAttribute(k_spread_gather<T, TS, TZ, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return;  // the launch error is reported by the caller's cudaGetLastError
        configured = smem;
    }
    int blocks = max_tiles < 152 * 4 ? max_tiles : 152 * 4;
    if (blocks < 1) blocks = 1;
    k_spread_gather<T, TS, TZ, TC><<<blocks, TS * TS * TZ, smem, s>>>(d, M, perm, mw, G, vol, scale, slot, ctab,
                                                                      list, count, cap, fu, fv, fw, ovf_list,
                                                                      ovf_count, next_tile);
}

template <typename T>
void launch_spread_gather(const Dims& d, int TS, int M, const int* perm, MarkerW<T> mw, const T* G, const double* vol,
                          double scale, const int* slot, const int* ctab, const int* list, const int* count,
                          int max_tiles, int cap, T* fu, T* fv, T* fw, int* ovf_list, int* ovf_count,
                          int* next_tile, cudaStream_t s, bool dfloat) {
    const bool flat = d.nz == 1;
#define AFMIB_SPREAD(TSV, TZV)                                                                                     \
    do {                                                                                                           \
        if (dfloat && sizeof(T) == sizeof(double))                                                                 \
            spread_launch<T, TSV, TZV, std::conditional_t<sizeof(T) == sizeof(double), dfl, T>>(                   \
                d, M, perm, mw, G, vol, scale, slot, ctab, list, count, max_tiles, cap, fu, fv, fw, ovf_list,      \
                ovf_count, next_tile, s);                                                                          \
        else                                                                                                       \
            spread_launch<T, TSV, TZV, T>(d, M, perm, mw, G, vol, scale, slot, ctab, list, count, max_tiles, cap, \
                                          fu, fv, fw, ovf_list, ovf_count, next_tile, s);                         \
    } while (0)
    if (TS == 8 && !flat) AFMIB_SPREAD(8, 8);
    else if (TS == 4 && !flat) AFMIB_SPREAD(4, 4);
    else if (TS == 8) AFMIB_SPREAD(8, 1);
    else AFMIB_SPREAD(4, 1);
#undef AFMIB_SPREAD
}

template <typename T, typename TF>
void launch_interp(const Dims& d, int M, const int* perm, MarkerW<T> mw, const TF* u, const TF* v, const TF* w, double* U,
                   cudaStream_t s) {
    if (M > 0) k_interp<T, TF><<<(M + 127) / 128, 128, 0, s>>>(d, M, perm, mw, u, v, w, U);
}

void launch_interp_dfl(const Dims& d, int M, const int* perm, MarkerW<double> mw, const double* u, const double* v,
                       const double* w, double* U, cudaStream_t s, const float* uh, const float* ul, const float* vh,
                       const float* vl, const float* wh, const float* wl) {
    if (M <= 0) return;
    const int blocks = (int)((4LL * M + kInterpDfBlock - 1) / kInterpDfBlock);
    if (uh && ul && vh && vl && wh && wl)
        k_interp_dfl<true><<<blocks, kInterpDfBlock, 0, s>>>(d, M, perm, mw, u, v, w, uh, ul, vh, vl, wh, wl, U);
    else
        k_interp_dfl<false><<<blocks, kInterpDfBlock, 0, s>>>(d, M, perm, mw, u, v, w, nullptr, nullptr, nullptr,
                                                               nullptr, nullptr, nullptr, U);
}

void launch_marker_axpy(int M, double* Xo, const double* Xi, const double* U, double c, cudaStream_t s) {
    if (M > 0) k_marker_axpy<<<(M + 255) / 256, 256, 0, s>>>(M, Xo, Xi, U, c);
}

#define AFMIB_IB_INST(T)                                                                                        \
    template void launch_springs<T>(int, const double*, const int*, const int*, double, T*, cudaStream_t);       \
    template void launch_springs_bending<T>(int, const double*, const int*, const int*, double, double, double*, T*, \
                                            cudaStream_t);                                                         \
    template void launch_marker_prep<T>(const Dims&, int, int, const double*, unsigned*, int*, MarkerW<T>, int*, \
                                        cudaStream_t, bool);                                                     \
    template size_t spread_smem_bytes<T>(int, int, int);                                                             \
    template void launch_spread_gather<T>(const Dims&, int, int, const int*, MarkerW<T>, const T*, const double*, \
                                          double, const int*, const int*, const int*, const int*, int, int, T*,  \
                                          T*, T*, int*, int*, int*, cudaStream_t, bool);                        \
    template void launch_interp<T, double>(const Dims&, int, const int*, MarkerW<T>, const double*, const double*, \
                                           const double*, double*, cudaStream_t);                               \
    template void launch_interp<T, float>(const Dims&, int, const int*, MarkerW<T>, const float*, const float*,  \
                                          const float*, double*, cudaStream_t);

AFMIB_IB_INST(double)
AFMIB_IB_INST(float)

}  // namespace afmib
