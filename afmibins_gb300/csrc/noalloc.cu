// Helmholtz CG that allocates nothing: afmib_helmholtz_cg_noalloc.
//
// Who needs it: callers that may not allocate device memory at the point of
// the call — code running inside a memory pool or arena that owns every
// cudaMalloc of the process, code running under a strict memory budget
// enforced by its host framework, or an inner loop where a cudaMalloc (an
// implicit device synchronisation) is not acceptable. They still pass their
// own x and b; the solve's own working vectors (r, p, q), the reduction
// partials, the reduction ticket and the CG scalars live in the file-scope
// array below, which the GPU holds from the moment the library's device code
// is loaded on it until the process exits.
//
// Limits and rules:
//  - at most kNoAllocMaxCells cells (64^3); larger grids are rejected;
//  - three-dimensional grids only (nx, ny, nz >= 2; a 2D grid is rejected);
//  - periodic domain (any component) or channel components 0 and 2 (u, w);
//    the channel v component needs a layout conversion buffer and is rejected;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current). Under
//    CUDA's lazy module loading (the default) that lookup is also what loads
//    the library's device code on the device, which reserves the array: the
//    first call therefore allocates, and may synchronise, once. A caller
//    whose budget starts later makes one warm-up call (or loads eagerly,
//    CUDA_MODULE_LOADING=EAGER) before it; every later call allocates
//    nothing. Make that first call before any stream capture;
//  - the address is kept per device for the life of the process: resetting a
//    device (cudaDeviceReset) while the library is in use is not supported;
//  - every call shares the one array, so calls that overlap on the GPU
//    (different streams or host threads at the same time) race and must not
//    be issued concurrently; the array keeps the last call's contents, and
//    each call clears the parts that must start at zero.
#include <cmath>

#include "afmib.h"
#include "kernels.h"

using namespace afmib;

namespace {

constexpr long long kNoAllocMaxCells = 64LL * 64LL * 64LL;
// r, p, q, reduction partials, CG scalars, and one slot for the ticket
constexpr long long kPartials = (long long)kMaxRedBlocks * kMaxRedVals;
constexpr long long kScalars = 16;
constexpr long long kScratchDoubles = 3 * kNoAllocMaxCells + kPartials + kScalars + 2;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
static double* g_scratch_addr[kMaxDevices] = {};

int scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return AFMIB_ERR_CUDA;
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return AFMIB_ERR_CUDA;
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return AFMIB_OK;
}

}  // namespace

extern "C" int afmib_helmholtz_cg_noalloc(int nx, int ny, int nz, int n, int bc, int comp, double scale, double tol,
                                          int max_iters, double* x, const double* b, int* iters, void* stream) {
    if (nx < 2 || ny < 2 || nz < 2 || comp < 0 || comp > 2 || !x || !b || !(tol > 0)) return AFMIB_ERR_ARG;
    if (bc != AFMIB_BC_PERIODIC && bc != AFMIB_BC_CHANNEL) return AFMIB_ERR_ARG;
    if (bc == AFMIB_BC_CHANNEL && comp == 1) return AFMIB_ERR_ARG;  // v needs a layout conversion buffer
    const long long N = (long long)nx * ny * nz;
    if (N > kNoAllocMaxCells) return AFMIB_ERR_CAPACITY;  // beyond the reserved array
    if (max_iters <= 0) max_iters = 1000;
    double* base = nullptr;
    const int rc = scratch_for_current_device(&base);
    if (rc != AFMIB_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const Dims d{nx, ny, nz, n > 0 ? n : nx, bc == AFMIB_BC_CHANNEL ? 1 : 0};
    double* r = base;
    double* p = base + N;
    double* q = base + 2 * N;
    RedScratch red{base + 3 * kNoAllocMaxCells, (unsigned*)(base + 3 * kNoAllocMaxCells + kPartials + kScalars)};
    double* cgs = base + 3 * kNoAllocMaxCells + kPartials;
    // the ticket must start at zero (a previous call may have been cut short)
    if (cudaMemsetAsync(red.ticket, 0, sizeof(unsigned), st) != cudaSuccess) return AFMIB_ERR_CUDA;
    double n0 = 0.0;
    launch_cg_init<double>(d, comp, scale, x, b, r, p, red, cgs, st);
    if (cudaGetLastError() != cudaSuccess) return AFMIB_ERR_CUDA;
    if (cudaMemcpyAsync(&n0, cgs, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return AFMIB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return AFMIB_ERR_CUDA;
    int it = 0;
    int status = AFMIB_OK;
    // the reference's loop, src/alg/cg.h:42-54, bounded by max_iters
    while (std::sqrt(n0) > tol) {
        if (!std::isfinite(n0)) { status = AFMIB_ERR_NAN; break; }
        if (it >= max_iters) { status = AFMIB_ERR_NOCONV; break; }
        launch_cg_apply<double>(d, comp, scale, p, q, red, cgs, st);
        launch_cg_update<double>(N, x, r, p, q, red, cgs, st);
        if (cudaMemcpyAsync(&n0, cgs, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return AFMIB_ERR_CUDA;
        launch_cg_direction<double>(N, p, r, cgs, st);
        if (cudaGetLastError() != cudaSuccess) return AFMIB_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return AFMIB_ERR_CUDA;
        ++it;
    }
    if (iters) *iters = it;
    return status;
}
