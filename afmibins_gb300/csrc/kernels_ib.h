// Immersed-boundary launch wrappers (kernels_ib.cu).
#pragma once

#include "kernels.h"

namespace afmib {

// Per-marker data computed once per marker configuration: wrapped cell,
// and for each axis a and face-offset variant v (0: integer positions, 1:
// half-integer) the first of the four faces relative to the cell and the
// four weights phi/n.
template <typename T>
struct MarkerW {
    int* cell;           // [M][3]
    signed char* dbase;  // [M][3][2]
    T* w;                // [M][3][2][4]
};

template <typename T>
void launch_springs(int M, const double* X, const int* nstart, const int* nidx, double k, T* G, cudaStream_t s);
// Springs plus bending: G = ks L X - kb L (L X), with Y (3M doubles) the
// workspace that receives L X; the bending term is the force of the discrete
// membrane energy kb/2 sum_i |(L X)_i|^2.
template <typename T>
void launch_springs_bending(int M, const double* X, const int* nstart, const int* nidx, double ks, double kb,
                            double* Y, T* G, cudaStream_t s);

// keys = tile * TS^2 TZ + cell-in-tile (TZ = TS, or 1 on a 2D grid), vals =
// marker index; flag set to 1 when a marker is within 2.5h of a channel wall,
// 2 on a NaN position.
template <typename T>
// df_weights (FP64 weights): sine and cosine in double-float on the FP32 pipe
// (df_sincospi) instead of the FP64 sincospi, weights within 2^-45 (the
// mixed form)
void launch_marker_prep(const Dims& d, int TS, int M, const double* X, unsigned* keys, int* vals, MarkerW<T> mw,
                        int* flag, cudaStream_t s, bool df_weights = false);

size_t radix_sort_temp_bytes(int n);
// Stable LSD sort of the low `bits` bits; returns which buffers hold the result.
void radix_sort_pairs(unsigned* keys, int* vals, unsigned* keys_alt, int* vals_alt, int n, int bits, unsigned* hist,
                      unsigned** keys_out, int** vals_out, cudaStream_t s);

void launch_tile_ranges(const unsigned* keys, int M, int cells_per_tile, int* tstart, int* tend, cudaStream_t s);
// slot[t] = storage slot of occupied tile t (or -1), occ[slot] = t; list of
// output tiles with a marker in their 3^3-tile neighbourhood.
void launch_active_tiles(int ntx, int nty, int ntz, int channel, const int* tstart, const int* tend, int* list,
                         int* count, int* slot, int* occ, int* occ_count, cudaStream_t s);
// ctab[slot][c]: first sorted position of local cell c of each occupied tile
void launch_cell_table(int TS, int TZ, const unsigned* keys, const int* tstart, const int* tend, const int* occ,
                       const int* occ_count, int max_occ, int* ctab, cudaStream_t s);

template <typename T>
size_t spread_smem_bytes(int TS, int TZ, int cap);
// f_c(face) = scale * sum_k (phi/n)^3 * vol_k * G_c,k over the active tiles
// (faces of the other tiles, and of active tiles whose neighbourhood holds no
// marker, are left untouched: the callers zero the fields first). A tile whose neighbourhood
// holds more than `cap` markers is appended to ovf_list (and left untouched)
// when ovf_list is given, else spread in chunks of `cap` markers (same
// result bits as one pass). Blocks take tiles from *next_tile, which must be
// zero at launch. dfloat (FP64 inputs): weight products and face sums in
// double-float on the FP32 pipe (relative 2^-44) instead of FP64.
template <typename T>
void launch_spread_gather(const Dims& d, int TS, int M, const int* perm, MarkerW<T> mw, const T* G, const double* vol,
                          double scale, const int* slot, const int* ctab, const int* list, const int* count,
                          int max_tiles, int cap, T* fu, T* fv, T* fw, int* ovf_list, int* ovf_count,
                          int* next_tile, cudaStream_t s, bool dfloat = false);

// U[c*M + k] = sum (phi/n)^3 u_c(face); perm (may be null) orders the threads.
// T: weight and arithmetic type, TF: field storage type
template <typename T, typename TF>
void launch_interp(const Dims& d, int M, const int* perm, MarkerW<T> mw, const TF* u, const TF* v, const TF* w, double* U,
                   cudaStream_t s);

// The FP64 interpolation in double-float on the FP32 pipe (axis-by-axis sums,
// relative error a few units of 2^-46 of the largest term): the mixed form.
// uh/ul, vh/vl, wh/wl (all given or none): the velocity's float pairs
// (hi + lo = u to 2^-46), read instead of splitting the FP64 values.
void launch_interp_dfl(const Dims& d, int M, const int* perm, MarkerW<double> mw, const double* u, const double* v,
                       const double* w, double* U, cudaStream_t s, const float* uh = nullptr,
                       const float* ul = nullptr, const float* vh = nullptr, const float* vl = nullptr,
                       const float* wh = nullptr, const float* wl = nullptr);

void launch_marker_axpy(int M, double* Xo, const double* Xi, const double* U, double c, cudaStream_t s);

}  // namespace afmib
