// afmib solver: host orchestration of the sm_103a kernels behind the C ABI
// declared in include/afmib.h.
//
// One solver owns the device-resident state of one simulation (velocity,
// projection potential, multigrid hierarchy, CG workspace, markers) and
// enqueues every kernel on one CUDA stream. Iterative loops keep their
// scalars on the device; the host reads one convergence scalar per
// iteration, exactly where the reference tests its stopping criterion.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "afmib.h"
#include "kernels.h"
#include "kernels_ib.h"
#include "kernels_adjoint.h"
#include "snapshot_io.h"

using namespace afmib;

template <typename T>
struct MGLevelT {
    Dims d;
    T *x, *b, *r;
    T* x2;       // ping-pong partner of x for the pipelined sweep (null where it does not apply)
    PipeCfg pc;  // pipelined-sweep launch shape (pc.FY == 0: per-colour launches)
};
typedef MGLevelT<double> MGLevel;

constexpr int kMaxInnerCycles = 8;  // longest FP32 inner V-cycle block of the mixed form

struct afmib_solver {
    afmib_config cfg{};
    Dims d{};
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::vector<void*> allocs;
    std::string err;
    afmib_stats stats{};

    // FP64 state on MAC faces (v padded to ny planes in channel mode)
    double *u = nullptr, *v = nullptr, *w = nullptr;
    double *uo[3] = {}, *adv[3] = {}, *rhs[3] = {}, *f[3] = {};
    // mixed form: Q(uold), the off-diagonal term of the viscous rows, kept by
    // the backward-Euler sub-step for the Crank-Nicolson right-hand side
    // (AFMIB_FUSED_RHS=0: each right-hand side and first defect apart)
    double* qo[3] = {};
    bool qo_valid = false;
    bool fused_rhs = true;
    // mixed form: the three viscous solves of a sub-step interleaved on two
    // streams, one component's FP32 correction beside the next component's
    // FP64 defect (AFMIB_HELM_OVERLAP=0: one solve after another). The
    // defects then run on a persistent grid of walk_blocks blocks (3 per SM,
    // AFMIB_HELM_WALK_BLOCKS) so that the corrections find free SM slots.
    bool helm_overlap = true;
    int walk_blocks = 0, walk_blocks_be = 0;  // the backward-Euler fused first defects (AFMIB_HELM_WALK_BLOCKS_BE)
    // the defects run on a stream of the device's highest priority (hi), so
    // that their persistent blocks take free SM slots before pending blocks
    // of the corrections on aux (measured no faster or slower than default
    // priority at 256^3: the defects are queued ahead of the corrections)
    cudaStream_t aux = nullptr, hi = nullptr;
    cudaEvent_t ev_def[3] = {}, ev_cor[3] = {}, ev_join = nullptr;
    float* d32c[3] = {};  // per-component defects; d32c[0] is d32
    // interleaved solves: after the first FP64 defect, the outer residual of
    // each viscous solve is kept as a double-float pair (d32c[c], rlo[c]) and
    // updated by r -= H e in double-float on the correction stream (an
    // HBM-bound pass fused with x += e) instead of re-evaluating b - H x with
    // the FP64 stencil (AFMIB_HELM_DF=0: FP64 defects); red2 is that
    // stream's reduction scratch
    bool helm_df = true;
    float* rlo[3] = {};
    RedScratch red2{};
    // the same for the pressure solve: after its first FP64 defect the
    // residual is the pair (lv32[0].b, plo), updated by r -= L e in
    // double-float at the end of each block of inner V-cycles, fused with
    // x += e (AFMIB_LAP_DF=0: an FP64 defect per block)
    bool lap_df = true;
    float* plo = nullptr;
    // mixed form: the FP64 spreading of the IB step computes its weight
    // products and face sums in double-float (relative 2^-44; the FP64 form
    // and the single-operator entry point stay FP64; AFMIB_SPREAD_DF=0: FP64)
    bool spread_df = true;
    // mixed form: the FP64 interpolation of the IB step in double-float too
    // (k_interp_dfl; AFMIB_INTERP_DF=0: FP64 arithmetic)
    bool interp_df = true;
    // mixed form: the FP32 velocity shadow (the FP32 advection's input) is
    // rounded to nearest by integer operations (AFMIB_SHADOW_ROUND=0:
    // truncated, a one-sided 2^-23 relative error)
    int round_shadow = 1;
    // mixed form: advection in FP64 from the FP64 velocity (AFMIB_ADVECT64=1)
    bool advect64 = false;
    // mixed form: the FP32 advection from the velocity's float pairs without
    // cancellation (k_advect_df; AFMIB_ADVECT_DF=0: the FP32 fluxes of the
    // rounded shadow, 1.0e-8 from the FP64 form after 100 steps at 256^3)
    bool advect_df = true;
    // mixed form: the first residuals of the viscous solves (BE pass with
    // Q(uold), CN from Q) in double-float on the FP32 pipe
    // (k_helm_rhs_be_defect_df, k_helm_cn_first_df; opt-in,
    // AFMIB_FIRST_DF=1: measured 56.36 against 56.49 IB steps/s for the FP64
    // passes at 256^3, which run beside the other stream's corrections)
    bool first_df = false;
    // mixed form: the divergence (with the sum of b) and the first pressure
    // defect (with the mean removal folded in) in double-float on the FP32
    // pipe; AFMIB_PROJ_DF=0 keeps the FP64 passes. At 256^3 the two run at
    // about the FP64 kernels' time (238 / 283 against 233 / 267 us: the
    // integer splits of the FP64 inputs make them issue-bound) and remove
    // the mean pass (104 us per projection). A double-float gradient update
    // measured slower (354 against 294 us) and is not used.
    bool proj_df = true;
    bool b_sum_ready = false;
    // mixed form: the double-float interpolation of the step's velocity reads
    // its float pairs (written by the projection) instead of splitting the
    // FP64 values (AFMIB_INTERP_PAIRS=0: splits)
    bool interp_pairs = true;
    // mixed form: the IB step's FP64 marker weights from double-float sines
    // and cosines on the FP32 pipe (df_sincospi) instead of the FP64
    // sincospi (AFMIB_PREP_DF=0: FP64)
    bool prep_df = true;  // scal[8] holds the sum of lv[0].b (from the divergence)
    // mixed form with the double-float residual: the Crank-Nicolson viscous
    // solves start from uold (the step's start velocity), whose residual
    // comes pointwise from the kept Q, instead of the current velocity
    // (AFMIB_CN_START_OLD=0: the current velocity and an FP64 stencil)
    bool cn_start_old = true;
    double *divb = nullptr, *walls = nullptr, *wallgrad = nullptr;
    double *cg_r = nullptr, *cg_p = nullptr, *cg_q = nullptr;
    double *tmp[3] = {};
    std::vector<MGLevel> lv;
    double *cw_p = nullptr, *cw_q = nullptr;

    // mixed form: FP32 inner workspaces (advection, forces, defects,
    // corrections, CG vectors, FP32 multigrid hierarchy) and the FP64 copy of
    // the coarsest level, which is solved in FP64
    bool mixed = false;
    float *adv32[3] = {}, *f32[3] = {}, *d32 = nullptr, *e32 = nullptr;
    float *u32 = nullptr, *v32 = nullptr, *w32 = nullptr;  // FP32 shadow of the velocity
    float *u32l = nullptr, *v32l = nullptr, *w32l = nullptr;  // the rest of each value's float pair
    float *cg32_r = nullptr, *cg32_p = nullptr, *cg32_q = nullptr, *cg32_p2 = nullptr;
    std::vector<MGLevelT<float>> lv32;
    double *cx64 = nullptr, *cb64 = nullptr, *cr64 = nullptr;
    // cap of V-cycles per FP32 inner solve, at most kMaxInnerCycles
    // (AFMIB_INNER_CYCLES); with the adaptive sizing below a long cap costs
    // nothing on the last correction (256^3 IB step: 3 -> 6 saved 2 FP64
    // defects per step)
    int inner_cycles = 6;
    // size each correction's inner solve from the per-cycle contraction seen
    // in the previous one: only the cycles that bring the defect below
    // tol / 2 (AFMIB_INNER_ADAPT=0: always inner_cycles)
    bool adapt_cycles = true;
    // The FP32 inner cycles only precondition the FP64 defect correction, so
    // they keep their own schedule: red-black sweeps over-relaxed by omega on
    // levels with nx >= 64 (AFMIB_INNER_OMEGA; 1: Gauss-Seidel) and (nu1, nu2)
    // sweeps around the coarse correction (AFMIB_INNER_NU=a,b). V(2,1) with
    // omega = 1.25 measured fastest at 256^3 (36.4 steps/s against 33.8 for
    // the FP64 cycles' V(2,2) Gauss-Seidel). The FP64 cycles keep the
    // configuration's nu1, nu2 and plain Gauss-Seidel.
    double inner_omega = 1.25;
    int inner_nu1 = 2, inner_nu2 = 1;
    // the same below the finest level (AFMIB_INNER_NU_COARSE=a,b)
    int inner_nu1c = 2, inner_nu2c = 1;
    double mg_rho = 0.0;        // measured per-cycle contraction (0: none yet)
    // pipelined red-black sweeps (AFMIB_SMOOTHER=pipe); the default is the
    // batched per-colour launches, measured faster at 256^3
    bool pipe_smoother = false;
    int pipe_min_nx = 64;       // smaller levels keep the per-colour launches (AFMIB_PIPE_MIN_NX)
    // mixed form: FP64-state defects by int64 block arithmetic instead of the
    // FP64 kernels (opt-in, AFMIB_BFP=1: measured no faster on GB300, the
    // integer form being instruction-bound at about the FP64 kernels' time)
    bool bfp_defects = false;
    // first multigrid level handled by the V-cycle tail (-1: none;
    // AFMIB_MG_TAIL=0), and the thread-block cluster it runs on (1: one
    // block)
    int tail_level = -1;
    int tail_cluster = 1;
    // mixed form: inner Helmholtz solves by fixed Jacobi sweeps where the
    // operator's diagonal dominance bounds them, as red-black Gauss-Seidel
    // sweeps (the default where the grid takes them: they contract as the
    // square of the Jacobi rate, two sweeps for four, 2.8 against 4.5 ms per
    // two 256^3 IB steps) or Jacobi sweeps; CG otherwise
    // (AFMIB_INNER_SOLVER=gs|jacobi|cg)
    bool jacobi_inner = true;
    bool gs_inner = true;
    // V-cycle blocks captured once into CUDA graphs and replayed (no host
    // interaction inside a V-cycle); not used while per-kernel profiling is on
    bool use_graphs = true;
    // passes over fields larger than L2 alternate their block order
    // (AFMIB_ALTERNATE=0: always index order); pass_rev is the last direction
    bool alternate = true;
    int pass_rev = 0;
    cudaGraphExec_t vg64 = nullptr, vg32[kMaxInnerCycles + 1] = {};
    long long vg64_launches = 0, vg32_launches[kMaxInnerCycles + 1] = {};
    bool spread64 = false, interp64 = false;  // mixed form: IB transfers in FP64
    // warm start of each projection from the potential of the previous
    // projection of the same sub-step type (0: BE, 1: CN); off in the FP64
    // form unless asked for, which keeps the reference's start from zero
    bool warm_start = false;
    double* phi_prev[2] = {nullptr, nullptr};
    bool phi_valid[2] = {false, false};
    // second-order start (AFMIB_WARM_EXTRAP=1): 2 phi_prev - phi_prev2
    bool warm_extrap = false;
    double* phi_prev2[2] = {nullptr, nullptr};
    bool phi_valid2[2] = {false, false};
    int proj_phase = -1;  // phase of the projection in progress (-1: none)
    RedScratch red{};
    double* scal = nullptr;   // device scalars: [0..4] CG, [8] sum, [9] sumsq, [16..17] adjoint scale
    double* hscal = nullptr;  // pinned mirror
    int* dflag = nullptr;     // device status flags [0] markers, [1] coarse solve, [3] pipelined smoother
    int* hflag = nullptr;
    bool half = false;

    // markers
    int M = 0, Mcap = 0, nnz_cap = 0;
    double *X = nullptr, *Xh = nullptr, *U1 = nullptr, *U2 = nullptr, *G = nullptr, *mvol = nullptr;
    double* Ybend = nullptr;  // L X (or L lamG in the adjoint) for the bending force
    int *nstart = nullptr, *nidx = nullptr;
    bool has_vol = false;
    unsigned *keys = nullptr, *keys2 = nullptr, *hist = nullptr;
    int *vals = nullptr, *vals2 = nullptr, *perm = nullptr;
    int TS = 0, TZ = 0, ntx = 0, nty = 0, ntz = 0, ntiles = 0;  // TZ: tile depth (TS; 1 on a 2D grid)
    int tile_cells() const { return TS * TS * TZ; }
    // tcount: [0] active output tiles, [1] occupied tiles, [2] tiles left to the large-capacity spreading pass,
    // [3], [4] the two passes' tile counters
    int *tstart = nullptr, *tend = nullptr, *tlist = nullptr, *tcount = nullptr, *tovf = nullptr;
    int *tslot = nullptr, *tocc = nullptr, *ctab = nullptr;
    int ctab_cap = 0;  // occupied tiles the cell table can hold
    MarkerW<double> mw{};
    MarkerW<float> mw32{};
    float* G32 = nullptr;
    bool nbr_symmetric = false;

    // trajectory with checkpoints for the reverse (adjoint) pass
    int traj_steps = 0, traj_every = 0;
    std::vector<double*> ck_vel, ck_X;                     // checkpoints: [3N], [3M]
    double *fin_vel = nullptr, *fin_X = nullptr;           // end state of the trajectory
    std::vector<double*> rec_u0, rec_uh, rec_X0, rec_Xh;   // one segment's forward record
    bool recording = false;
    int rec_j = 0;
    int traj_M = 0;
    double* adj_f[4] = {};                                 // L, A, T, R: [3N] each
    double *lamX = nullptr, *lamXh = nullptr, *mbar1 = nullptr, *mbar2 = nullptr, *lamG = nullptr, *Gtmp = nullptr,
           *Ubuf = nullptr, *dkp = nullptr;

    // per-kernel event timing (afmib_profile_*): ranges recorded around each
    // launch while enabled, resolved at the next synchronisation
    struct ProfEntry { const char* name; long long launches; double ms; double bytes; };
    struct ProfPending { int id; cudaEvent_t a, b; double bytes; };
    bool prof = false;
    std::vector<ProfEntry> prof_tab;
    std::vector<ProfPending> prof_pend;
    std::vector<cudaEvent_t> prof_pool;

    int fail(int code, const std::string& msg) {
        err = msg;
        return code;
    }
    long long N() const { return d.ncell(); }
    long long nxz() const { return (long long)d.nx * d.nz; }
    long long nv_user() const { return d.channel ? (long long)d.nx * (d.ny - 1) * d.nz : N(); }
    double s_plus() const { return cfg.mu * cfg.dt / (2 * cfg.rho); }
    double s_minus() const { return -cfg.mu * cfg.dt / (2 * cfg.rho); }
};

namespace {

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return s->fail(AFMIB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CKL()                                                                                 \
    do {                                                                                      \
        cudaError_t e_ = cudaGetLastError();                                                  \
        if (e_ != cudaSuccess) return s->fail(AFMIB_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
    } while (0)

#define TRY(expr)               \
    do {                        \
        int rc_ = (expr);       \
        if (rc_ != AFMIB_OK) return rc_; \
    } while (0)

template <typename T>
int dalloc(afmib_solver* s, T** p, size_t count) {
    void* q = nullptr;
    CK(cudaMalloc(&q, (count > 0 ? count : 1) * sizeof(T)));
    s->allocs.push_back(q);
    *p = (T*)q;
    return AFMIB_OK;
}

bool is_even(int v) { return v % 2 == 0; }

// --- layout conversions between the caller's v (ny-1 interior planes in
// channel mode) and the padded device v (ny planes, plane 0 = wall) ---------
int v_in(afmib_solver* s, double* dev_padded, const double* user) {
    const Dims& d = s->d;
    if (!d.channel) {
        CK(cudaMemcpyAsync(dev_padded, user, s->N() * sizeof(double), cudaMemcpyDefault, s->st));
        return AFMIB_OK;
    }
    CK(cudaMemsetAsync(dev_padded, 0, s->N() * sizeof(double), s->st));
    CK(cudaMemcpy2DAsync(dev_padded + d.nx, (size_t)d.nx * d.ny * sizeof(double), user,
                         (size_t)d.nx * (d.ny - 1) * sizeof(double), (size_t)d.nx * (d.ny - 1) * sizeof(double),
                         d.nz, cudaMemcpyDefault, s->st));
    return AFMIB_OK;
}

int v_out(afmib_solver* s, double* user, const double* dev_padded) {
    const Dims& d = s->d;
    if (!d.channel) {
        CK(cudaMemcpyAsync(user, dev_padded, s->N() * sizeof(double), cudaMemcpyDefault, s->st));
        return AFMIB_OK;
    }
    CK(cudaMemcpy2DAsync(user, (size_t)d.nx * (d.ny - 1) * sizeof(double), dev_padded + d.nx,
                         (size_t)d.nx * d.ny * sizeof(double), (size_t)d.nx * (d.ny - 1) * sizeof(double), d.nz,
                         cudaMemcpyDefault, s->st));
    return AFMIB_OK;
}

int copy_in(afmib_solver* s, double* dst, const double* src, long long n) {
    if (src) CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, s->st));
    else CK(cudaMemsetAsync(dst, 0, n * sizeof(double), s->st));
    return AFMIB_OK;
}

int copy_out(afmib_solver* s, double* dst, const double* src, long long n) {
    if (dst) CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, s->st));
    return AFMIB_OK;
}

void prof_flush(afmib_solver* s);

int sync(afmib_solver* s) {
    CK(cudaStreamSynchronize(s->st));
    if (s->prof) prof_flush(s);
    return AFMIB_OK;
}

// ---- per-kernel profiling -------------------------------------------------
enum ProfId {
    P_ADVECT, P_HELM_RHS, P_CG_INIT, P_CG_APPLY, P_CG_UPDATE, P_CG_DIR, P_RBGS, P_RESID, P_RESID_NORM,
    P_RESTRICT, P_PROLONG, P_COARSE, P_DIV, P_GRAD_SUB, P_MEAN, P_WALL, P_SPRINGS, P_PREP, P_SORT,
    P_TILES, P_SPREAD, P_INTERP, P_MARKER, P_HELM_DEFECT, P_LAP_DEFECT, P_CORRECT, P_ADJ_ADVECT, P_ADJ_MARKER,
    P_RBGS0, P_RESID0, P_RESTRICT0, P_PROLONG0, P_CG_DIRAPPLY, P_TAIL, P_JACOBI, P_HELM_UPDATE, P_LAP_UPDATE,
    P_RESID_RESTRICT0, P_RESID_RESTRICT, P_COUNT
};
const char* kProfNames[P_COUNT] = {
    "advect", "helm_rhs", "cg_init", "cg_apply", "cg_update", "cg_direction", "mg_rbgs", "mg_residual",
    "mg_residual_norm", "mg_restrict", "mg_prolong_add", "mg_coarse_cg", "div", "grad_sub", "mean_removal",
    "wall_update", "springs", "marker_prep", "radix_sort", "tile_bins", "spread_gather", "interp", "marker_update",
    "helm_defect_fp64", "lap_defect_first", "add_correction_fp64", "advect_adjoint", "marker_adjoint",
    "mg_rbgs_fine", "mg_residual_fine", "mg_restrict_fine", "mg_prolong_add_fine", "cg_dir_apply", "mg_coarse_tail",
    "helm_inner_sweep_fp32", "helm_update_df", "lap_update_df", "mg_resid_restrict_fine", "mg_resid_restrict"};

cudaEvent_t prof_event(afmib_solver* s) {
    if (!s->prof_pool.empty()) {
        cudaEvent_t e = s->prof_pool.back();
        s->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_flush(afmib_solver* s) {
    for (auto& p : s->prof_pend) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            auto& e = s->prof_tab[p.id];
            e.launches++;
            e.ms += ms;
            e.bytes += p.bytes;
        }
        s->prof_pool.push_back(p.a);
        s->prof_pool.push_back(p.b);
    }
    s->prof_pend.clear();
}

// Brackets one (or a fixed group of) kernel launch(es) with events when
// profiling is on; counts the launches either way.
// q: the stream the launches go to (default: the solver's stream).
struct ProfScope {
    afmib_solver* s;
    int id;
    double bytes;
    cudaStream_t q;
    cudaEvent_t a = nullptr;
    ProfScope(afmib_solver* s_, int id_, double bytes_, int launches = 1, cudaStream_t q_ = nullptr)
        : s(s_), id(id_), bytes(bytes_), q(q_ ? q_ : s_->st) {
        s->stats.kernel_launches += launches;
        if (s->prof) {
            a = prof_event(s);
            cudaEventRecord(a, q);
        }
    }
    ~ProfScope() {
        if (s->prof && a) {
            cudaEvent_t b = prof_event(s);
            cudaEventRecord(b, q);
            s->prof_pend.push_back({id, a, b, bytes});
        }
    }
};

// read n doubles of the device scalar block into the pinned mirror
int read_scalars(afmib_solver* s, int first, int n) {
    CK(cudaMemcpyAsync(s->hscal + first, s->scal + first, n * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    return sync(s);
}

// ---------------------------------------------------------------------------
// CG, src/alg/cg.h:32-56 (absolute 2-norm stop, warm start from x), bounded.
// Algorithmic bytes per launch (s = 8): init 4N s, apply 2N s, update 6N s,
// direction 3N s.
// ---------------------------------------------------------------------------
int cg_solve(afmib_solver* s, int comp, double scale, double* x, const double* b, int* iters) {
    const Dims& d = s->d;
    const long long N = s->N();
    const double Ns = (double)N * sizeof(double);
    {
        ProfScope ps(s, P_CG_INIT, 4 * Ns);
        launch_cg_init<double>(d, comp, scale, x, b, s->cg_r, s->cg_p, s->red, s->scal, s->st);
    }
    CKL();
    TRY(read_scalars(s, 0, 1));
    int it = 0;
    int status = AFMIB_OK;
    while (std::sqrt(s->hscal[0]) > s->cfg.tol) {
        if (!std::isfinite(s->hscal[0])) { status = s->fail(AFMIB_ERR_NAN, "CG residual is not finite"); break; }
        if (it >= s->cfg.max_cg_iters) { status = s->fail(AFMIB_ERR_NOCONV, "CG iteration cap reached"); break; }
        {
            ProfScope ps(s, P_CG_APPLY, 2 * Ns);
            launch_cg_apply<double>(d, comp, scale, s->cg_p, s->cg_q, s->red, s->scal, s->st);
        }
        {
            ProfScope ps(s, P_CG_UPDATE, 6 * Ns);
            launch_cg_update<double>(N, x, s->cg_r, s->cg_p, s->cg_q, s->red, s->scal, s->st);
        }
        CK(cudaMemcpyAsync(s->hscal, s->scal, sizeof(double), cudaMemcpyDeviceToHost, s->st));
        {
            ProfScope ps(s, P_CG_DIR, 3 * Ns);
            launch_cg_direction<double>(N, s->cg_p, s->cg_r, s->scal, s->st);
        }
        CKL();
        TRY(sync(s));
        ++it;
    }
    s->stats.cg_iters += it;
    s->stats.last_cg_norm = std::sqrt(s->hscal[0]);
    if (iters) *iters = it;
    return status;
}

// ---------------------------------------------------------------------------
// Multigrid, src/mg/solver.h. V(nu1, nu2) cycles with red-black Gauss–Seidel,
// the reference's full-weighting restriction and trilinear prolongation, and
// the coarsest level solved by mean removal + CG (src/mg/solver.h:264-271).
// Algorithmic bytes: a full red+black sweep reads x and b and writes x once
// (3N s, so 1.5N s per colour launch); residual 3N s; restriction N s + N/8 s;
// prolongation-add 2N s + N/8 s.
// ---------------------------------------------------------------------------
template <typename T>
std::vector<MGLevelT<T>>& levels(afmib_solver* s);
template <>
std::vector<MGLevelT<double>>& levels<double>(afmib_solver* s) { return s->lv; }
template <>
std::vector<MGLevelT<float>>& levels<float>(afmib_solver* s) { return s->lv32; }

// Block order of the next pass over a field of level d (block_at): passes
// over arrays of more than 32 MB (the 126 MB L2 holds about two of them)
// alternate, so that each starts on the rows the previous one left in L2.
// Measured at 256^3: fine-level red-black sweeps 7.11 -> 6.04 ms per two IB
// steps with the black sweeps reversed.
int pass_dir(afmib_solver* s, const Dims& d, size_t elem) {
    if (!s->alternate || (double)d.ncell() * (double)elem < 32.0 * (1 << 20)) return 0;
    s->pass_rev ^= 1;
    return s->pass_rev;
}

// from_zero: x starts at zero and its contents are not (the first colour
// writes both colours: launch_rbgs_from_zero)
template <typename T>
int smooth(afmib_solver* s, MGLevelT<T>& L, int sweeps, bool from_zero = false) {
    const double Ns = (double)L.d.ncell() * sizeof(T);
    const int id = L.d.nx == s->d.nx ? P_RBGS0 : P_RBGS;  // finest level kept apart in the profile
    const double omega = sizeof(T) == sizeof(float) ? s->inner_omega : 1.0;
    int j = 0;
    const bool pipe = L.x2 && s->pipe_smoother && L.pc.FY && omega == 1.0;
    if (from_zero && (pipe || sweeps < 1)) {
        CK(cudaMemsetAsync(L.x, 0, L.d.ncell() * sizeof(T), s->st));
        from_zero = false;
    }
    if (pipe) {
        // pairs of pipelined sweeps, x -> x2 -> x
        for (; j + 2 <= sweeps; j += 2) {
            {
                ProfScope ps(s, id, 3 * Ns);
                launch_rbgs_pipe<T>(L.d, L.pc, L.x, L.x2, L.b, s->dflag + 3, s->st);
            }
            {
                ProfScope ps(s, id, 3 * Ns);
                launch_rbgs_pipe<T>(L.d, L.pc, L.x2, L.x, L.b, s->dflag + 3, s->st);
            }
        }
    }
    for (; j < sweeps; ++j) {
        if (from_zero && j == 0) {
            ProfScope ps(s, id, 1.5 * Ns);
            launch_rbgs_from_zero<T>(L.d, L.x, L.b, s->st, omega, pass_dir(s, L.d, sizeof(T)));
        } else {
            ProfScope ps(s, id, 1.5 * Ns);
            launch_rbgs<T>(L.d, 0, L.x, L.b, s->st, omega, pass_dir(s, L.d, sizeof(T)));
        }
        {
            ProfScope ps(s, id, 1.5 * Ns);
            launch_rbgs<T>(L.d, 1, L.x, L.b, s->st, omega, pass_dir(s, L.d, sizeof(T)));
        }
    }
    CKL();
    return AFMIB_OK;
}

// coarsest level: FP64 solve (the FP32 hierarchy hands its level to FP64)
int coarse(afmib_solver* s, MGLevelT<double>& L) {
    ProfScope ps(s, P_COARSE, 3.0 * L.d.ncell() * sizeof(double));
    launch_coarse_solve<double>(L.d, L.x, L.b, L.r, s->cw_p, s->cw_q, s->cfg.tol, s->cfg.max_cg_iters, s->dflag + 1,
                                s->st);
    return AFMIB_OK;
}
int coarse(afmib_solver* s, MGLevelT<float>& L) {
    const long long n = L.d.ncell();
    ProfScope ps(s, P_COARSE, 3.0 * n * sizeof(double), 3);
    launch_convert<double, float>(n, s->cb64, L.b, s->st);
    launch_coarse_solve<double>(L.d, s->cx64, s->cb64, s->cr64, s->cw_p, s->cw_q, s->cfg.tol, s->cfg.max_cg_iters,
                                s->dflag + 1, s->st);
    launch_convert<float, double>(n, L.x, s->cx64, s->st);
    return AFMIB_OK;
}

// the coarse V-cycle below level l in one block or one cluster (k_vcycle_tail)
template <typename T>
int vcycle_tail(afmib_solver* s, size_t l) {
    auto& lv = levels<T>(s);
    TailLevels<T> a{};
    a.nlev = (int)(lv.size() - l);
    a.nu1 = sizeof(T) == sizeof(float) ? s->inner_nu1c : s->cfg.nu1;
    a.nu2 = sizeof(T) == sizeof(float) ? s->inner_nu2c : s->cfg.nu2;
    a.maxit = s->cfg.max_cg_iters;
    a.tol = s->cfg.tol;
    for (int k = 0; k < a.nlev; ++k) {
        a.d[k] = lv[l + k].d;
        a.x[k] = lv[l + k].x;
        a.b[k] = lv[l + k].b;
        a.r[k] = lv[l + k].r;
    }
    a.cx64 = s->cx64;
    a.cb64 = s->cb64;
    a.cr64 = s->cr64;
    a.cw_p = s->cw_p;
    a.cw_q = s->cw_q;
    a.status = s->dflag + 1;
    ProfScope ps(s, P_TAIL, 0.0);
    launch_vcycle_tail<T>(a, s->st, s->tail_cluster);
    CKL();
    return AFMIB_OK;
}

// x_zero: level l's x starts at zero, its contents not yet cleared
template <typename T>
int vcycle(afmib_solver* s, size_t l, bool x_zero = false) {
    auto& lv = levels<T>(s);
    MGLevelT<T>& L = lv[l];
    const double Ns = (double)L.d.ncell() * sizeof(T);
    const bool last = l + 1 == lv.size();
    if (x_zero && ((s->tail_level >= 0 && l == (size_t)s->tail_level) || last))
        CK(cudaMemsetAsync(L.x, 0, L.d.ncell() * sizeof(T), s->st));
    if (s->tail_level >= 0 && l == (size_t)s->tail_level) return vcycle_tail<T>(s, l);
    if (last) {
        TRY(coarse(s, L));
        CKL();
        return AFMIB_OK;
    }
    const bool fine = l == 0;
    TRY(smooth(s, L, sizeof(T) == sizeof(float) ? (fine ? s->inner_nu1 : s->inner_nu1c) : s->cfg.nu1, x_zero));
    MGLevelT<T>& C = lv[l + 1];
    if (resid_restrict_fused_ok(L.d, sizeof(T), L.x, L.b, C.b, C.x)) {
        // x, b read; coarse b and x written (the fine residual stays on chip)
        ProfScope ps(s, fine ? P_RESID_RESTRICT0 : P_RESID_RESTRICT, 2 * Ns + 2 * Ns / 8);
        launch_resid_restrict<T>(L.d, C.b, C.x, L.x, L.b, s->st, pass_dir(s, L.d, sizeof(T)));
    } else {
        {
            ProfScope ps(s, fine ? P_RESID0 : P_RESID, 3 * Ns);
            launch_residual<T>(L.d, L.r, L.x, L.b, nullptr, nullptr, s->st, pass_dir(s, L.d, sizeof(T)));
        }
        {
            // the coarse iterate starts from zero: set in the same pass
            ProfScope ps(s, fine ? P_RESTRICT0 : P_RESTRICT, Ns + Ns / 8 + Ns / 8);
            launch_restrict<T>(L.d, C.b, L.r, s->st, pass_dir(s, L.d, sizeof(T)), C.x);
        }
    }
    CKL();
    TRY(vcycle<T>(s, l + 1));
    {
        ProfScope ps(s, fine ? P_PROLONG0 : P_PROLONG, 2 * Ns + Ns / 8);
        launch_prolong_add<T>(L.d, L.x, C.x, s->st, pass_dir(s, L.d, sizeof(T)));
    }
    TRY(smooth(s, L, sizeof(T) == sizeof(float) ? (fine ? s->inner_nu2 : s->inner_nu2c) : s->cfg.nu2));
    return AFMIB_OK;
}

// phi for the start of a projection: the previous potential of the same
// sub-step type, or zero
int initial_potential(afmib_solver* s) {
    MGLevel& L = s->lv[0];
    const long long N = L.d.ncell();
    const int ph = s->proj_phase;
    if (s->warm_start && ph >= 0 && s->phi_valid[ph] && s->warm_extrap && s->phi_valid2[ph])
        launch_lincomb<double>(N, L.x, 2.0, s->phi_prev[ph], -1.0, s->phi_prev2[ph], s->st);
    else if (s->warm_start && ph >= 0 && s->phi_valid[ph])
        CK(cudaMemcpyAsync(L.x, s->phi_prev[ph], N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    else
        CK(cudaMemsetAsync(L.x, 0, N * sizeof(double), s->st));
    return AFMIB_OK;
}

// Capture `body` on the solver's stream into an executable graph.
template <typename F>
int capture_graph(afmib_solver* s, cudaGraphExec_t* exec, long long* launches, F body) {
    const long long l0 = s->stats.kernel_launches;
    CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    const int rc = body();
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->st, &g);
    if (rc != AFMIB_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return s->fail(AFMIB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    const cudaError_t e2 = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return s->fail(AFMIB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e2));
    *launches = s->stats.kernel_launches - l0;
    s->stats.kernel_launches = l0;  // recorded, not run
    return AFMIB_OK;
}

void drop_graphs(afmib_solver* s) {
    if (s->vg64) cudaGraphExecDestroy(s->vg64);
    s->vg64 = nullptr;
    for (auto& g : s->vg32) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// one FP64 V-cycle on level 0 (graph replay when possible)
int vcycle64_top(afmib_solver* s) {
    if (s->prof || !s->use_graphs) return vcycle<double>(s, 0);
    if (!s->vg64) TRY(capture_graph(s, &s->vg64, &s->vg64_launches, [&]() { return vcycle<double>(s, 0); }));
    CK(cudaGraphLaunch(s->vg64, s->st));
    s->stats.kernel_launches += s->vg64_launches;
    return AFMIB_OK;
}

// the FP32 inner solve of one defect-correction step: x32 = 0, ncyc
// V-cycles on L e = r, phi += e (graph replay when possible, one graph per
// cycle count)
// the pressure solve keeps its outer residual as a double-float pair
bool lap_df_on(const afmib_solver* s) { return s->lap_df && s->plo && !s->bfp_defects; }

// One block of ncyc FP32 V-cycles from zero on the residual in lv32[0].b,
// then x += e, and with lap_df_on also r -= L e with its norm in scal[9].
int inner_vcycles32(afmib_solver* s, int ncyc) {
    MGLevel& L = s->lv[0];
    MGLevelT<float>& L32 = s->lv32[0];
    const long long N = L.d.ncell();
    auto body = [&](int nc) {
        return [&, nc]() -> int {
            // the first cycle's first colour starts the correction from zero
            for (int k = 0; k < nc; ++k) TRY(vcycle<float>(s, 0, k == 0));
            if (lap_df_on(s)) {
                ProfScope ps(s, P_LAP_UPDATE, (double)N * (8 + 4 + 8 + 8 + 8 + 4));
                launch_lap_update_df(L.d, L.x, L32.x, L32.b, s->plo, s->red, s->scal + 9, s->st);
            } else {
                ProfScope ps(s, P_CORRECT, (double)N * (8 + 4 + 8));
                launch_add_correction<float>(N, L.x, L32.x, s->st);
            }
            CKL();
            return AFMIB_OK;
        };
    };
    if (s->prof || !s->use_graphs) return body(ncyc)();
    // every block length is captured at the first use of any: a length first
    // needed later (the adaptive sizing picks them as the residuals go) would
    // pay for its capture and instantiation inside a running time step
    if (!s->vg32[ncyc])
        for (int k = 1; k <= s->inner_cycles; ++k)
            if (!s->vg32[k]) TRY(capture_graph(s, &s->vg32[k], &s->vg32_launches[k], body(k)));
    CK(cudaGraphLaunch(s->vg32[ncyc], s->st));
    s->stats.kernel_launches += s->vg32_launches[ncyc];
    return AFMIB_OK;
}

// Solve L x = b on level 0 (b in lv[0].b, destroyed; x in lv[0].x), the
// reference's solve loop: remove the mean of b, then cycle until
// RMS(b - L x) <= tol (src/mg/solver.h:218-237).
int mg_solve(afmib_solver* s, int* cycles) {
    MGLevel& L = s->lv[0];
    const long long N = L.d.ncell();
    const double Ns = (double)N * sizeof(double);
    {
        ProfScope ps(s, P_MEAN, 3 * Ns, 2);
        launch_sum<double>(N, L.b, s->red, s->scal + 8, s->st);
        launch_sub_scalar_scaled<double>(N, L.b, s->scal + 8, 1.0 / (double)N, s->st);
    }
    TRY(initial_potential(s));
    CK(cudaMemsetAsync(s->dflag + 1, 0, sizeof(int), s->st));
    int status = AFMIB_OK;
    int c = 0;
    if (s->lv.size() == 1) {
        TRY(vcycle<double>(s, 0));
    } else {
        for (;;) {
            {
                ProfScope ps(s, P_RESID_NORM, 3 * Ns);
                launch_residual<double>(L.d, L.r, L.x, L.b, &s->red, s->scal + 9, s->st);
            }
            CKL();
            TRY(read_scalars(s, 9, 1));
            const double rms = std::sqrt(s->hscal[9]) / std::sqrt((double)N);
            s->stats.last_mg_rms = rms;
            if (!std::isfinite(rms)) { status = s->fail(AFMIB_ERR_NAN, "multigrid residual is not finite"); break; }
            if (rms <= s->cfg.tol) break;
            if (c >= s->cfg.max_mg_cycles) { status = s->fail(AFMIB_ERR_NOCONV, "multigrid cycle cap reached"); break; }
            TRY(vcycle64_top(s));
            ++c;
        }
    }
    CK(cudaMemcpyAsync(s->hflag + 1, s->dflag + 1, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(s->hflag + 3, s->dflag + 3, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    TRY(sync(s));
    if (s->hflag[3] != 0) return s->fail(AFMIB_ERR_CUDA, "pipelined smoother: a row copy did not complete in time");
    if (status == AFMIB_OK && s->hflag[1] != 0) status = s->fail(AFMIB_ERR_NOCONV, "coarsest-level CG did not converge");
    s->stats.mg_cycles += c;
    if (cycles) *cycles = c;
    return status;
}

// ---------------------------------------------------------------------------
// Mixed form. FP64 defect correction around FP32 inner solves: the residual
// of the FP64 iterate is evaluated in FP64 and handed to the FP32 solver as an
// FP32 defect; the FP32 correction is added to the FP64 iterate. The stopping
// tests are the reference's (CG: ||r||_2 <= tol, MG: RMS(r) <= tol) on the
// FP64 residual, so the converged iterate has the FP64 form's accuracy.
// ---------------------------------------------------------------------------
int cg_inner32(afmib_solver* s, int comp, double scale, double rel_tol, int* iters) {
    const Dims& d = s->d;
    const long long N = s->N();
    const double Ns = (double)N * sizeof(float);
    {
        ProfScope ps(s, P_CG_INIT, 4 * Ns);
        launch_cg_init_zero<float>(N, s->d32, s->e32, s->cg32_r, s->cg32_p, s->red, s->scal, s->st);
    }
    CKL();
    TRY(read_scalars(s, 0, 1));
    const double stop = rel_tol * std::sqrt(s->hscal[0]);
    int it = 0;
    // the direction update of iteration k is folded into the apply of k+1
    // (p and cg32_p2 alternate)
    float* p = s->cg32_p;
    float* pn = s->cg32_p2;
    while (std::sqrt(s->hscal[0]) > stop && it < s->cfg.max_cg_iters) {
        if (!std::isfinite(s->hscal[0])) return s->fail(AFMIB_ERR_NAN, "inner CG residual is not finite");
        if (it == 0) {
            ProfScope ps(s, P_CG_APPLY, 2 * Ns);
            launch_cg_apply<float>(d, comp, scale, p, s->cg32_q, s->red, s->scal, s->st);
        } else {
            ProfScope ps(s, P_CG_DIRAPPLY, 4 * Ns);
            launch_cg_dir_apply<float>(d, comp, scale, p, s->cg32_r, pn, s->cg32_q, s->red, s->scal, s->st);
            std::swap(p, pn);
        }
        {
            ProfScope ps(s, P_CG_UPDATE, 6 * Ns);
            launch_cg_update<float>(N, s->e32, s->cg32_r, p, s->cg32_q, s->red, s->scal, s->st);
        }
        CK(cudaMemcpyAsync(s->hscal, s->scal, sizeof(double), cudaMemcpyDeviceToHost, s->st));
        CKL();
        TRY(sync(s));
        ++it;
    }
    s->stats.cg_iters += it;
    if (iters) *iters = it;
    return AFMIB_OK;
}

// Jacobi sweeps for a relative reduction rel_tol of the inner Helmholtz
// solve, or -1 when CG should be used. For the implicit operator (scale < 0)
// H is strictly diagonally dominant: the Jacobi iteration contracts the
// max-norm error by rho = k|off| / (1 + k|off|) per sweep (k = 6, 4 in 2D;
// the channel wall rows contract faster). The outer loop measures the 2-norm
// of the residual, and the defects concentrate near the membrane (their
// max/RMS ratio is large), so the sweeps aim at rel_tol / 10 in the max
// norm: ceil(log(rel_tol / 10) / log(rho)) sweeps from zero (measured at
// 256^3: one sweep fewer costs a third defect-correction step per solve,
// one more costs a sweep per solve for nothing).
int jacobi_sweeps(const Dims& d, double scale, double rel_tol) {
    if (!(scale < 0)) return -1;
    const double off = -scale * (double)d.n * (double)d.n, k = d.nz == 1 ? 4.0 : 6.0;
    const double rho = k * off / (1.0 + k * off);
    if (!(rho > 0) || !(rho < 1)) return -1;
    int sweeps = (int)std::ceil(std::log(rel_tol * 1e-1) / std::log(rho));
    if (const char* e = std::getenv("AFMIB_JACOBI_SWEEPS")) sweeps = std::atoi(e);
    return sweeps >= 1 && sweeps <= 10 ? sweeps : -1;
}

// red-black Gauss-Seidel sweeps for the same reduction (rate rho^2 per sweep)
int gs_sweeps(const Dims& d, double scale, double rel_tol) {
    const int j = jacobi_sweeps(d, scale, rel_tol);
    if (j < 0) return -1;
    const double off = -scale * (double)d.n * (double)d.n, k = d.nz == 1 ? 4.0 : 6.0;
    const double rho = k * off / (1.0 + k * off);
    int sweeps = std::max(1, (int)std::ceil(std::log(rel_tol * 1e-1) / std::log(rho * rho)));
    if (const char* e = std::getenv("AFMIB_GS_SWEEPS")) sweeps = std::atoi(e);
    return sweeps >= 1 && sweeps <= 10 ? sweeps : -1;
}

// FP32 inner solve by red-black Gauss-Seidel sweeps in place on e32 from
// zero; false when the grid does not take the kernel (nothing launched)
bool gs_inner32(afmib_solver* s, int comp, double scale, int sweeps) {
    const long long N = s->N();
    for (int j = 0; j < sweeps; ++j)
        for (int color = 0; color < 2; ++color) {
            ProfScope ps(s, P_JACOBI, (double)N * 4 * 1.5);
            if (!launch_helm_rbgs<float>(s->d, comp, scale, color, j == 0 && color == 0, s->e32, s->d32, s->st,
                                         pass_dir(s, s->d, sizeof(float))))
                return false;
        }
    return true;
}

// FP32 inner solve by fixed Jacobi sweeps: e32 = H^-1 d32 to rel_tol
int jacobi_inner32(afmib_solver* s, int comp, double scale, int sweeps) {
    const long long N = s->N();
    float* bufs[2] = {s->e32, s->cg32_p};
    for (int j = 0; j < sweeps; ++j) {
        ProfScope ps(s, P_JACOBI, (double)N * 4 * (j == 0 ? 2 : 3));
        float* out = bufs[(sweeps - 1 - j) % 2];
        const float* in = j == 0 ? nullptr : bufs[(sweeps - j) % 2];
        launch_helm_jacobi<float>(s->d, comp, scale, in, out, s->d32, s->st, pass_dir(s, s->d, sizeof(float)));
    }
    CKL();
    return AFMIB_OK;
}

// r0_ready: the first defect (d32, its squared norm in scal[10]) is already
// computed for this x and b
int helm_solve_mixed(afmib_solver* s, int comp, double scale, double* x, const double* b, bool r0_ready = false) {
    const long long N = s->N();
    int outer = 0;
    for (;;) {
        if (!(r0_ready && outer == 0)) {
            ProfScope ps(s, P_HELM_DEFECT, (double)N * (8 + 8 + 4));
            if (s->bfp_defects)
                launch_helm_defect_bfp(s->d, comp, scale, x, b, s->d32, s->red, s->scal + 10, s->st);
            else
                launch_helm_defect<float>(s->d, comp, scale, x, b, s->d32, s->red, s->scal + 10, s->st);
        }
        CKL();
        TRY(read_scalars(s, 10, 1));
        const double nr = std::sqrt(s->hscal[10]);
        s->stats.last_cg_norm = nr;
        if (!std::isfinite(nr)) return s->fail(AFMIB_ERR_NAN, "Helmholtz residual is not finite");
        if (nr <= s->cfg.tol) break;
        if (outer >= s->cfg.max_mg_cycles) return s->fail(AFMIB_ERR_NOCONV, "defect-correction cap reached (Helmholtz)");
        const int gsw = s->gs_inner ? gs_sweeps(s->d, scale, s->cfg.inner_tol) : -1;
        const int sweeps = s->jacobi_inner ? jacobi_sweeps(s->d, scale, s->cfg.inner_tol) : -1;
        if (gsw > 0 && gs_inner32(s, comp, scale, gsw)) {
        } else if (sweeps > 0) {
            TRY(jacobi_inner32(s, comp, scale, sweeps));
        } else {
            TRY(cg_inner32(s, comp, scale, s->cfg.inner_tol, nullptr));
        }
        CKL();
        {
            ProfScope ps(s, P_CORRECT, (double)N * (8 + 4 + 8));
            launch_add_correction<float>(N, x, s->e32, s->st);
        }
        CKL();
        ++outer;
    }
    s->stats.outer_iters += outer;
    return AFMIB_OK;
}

// The three viscous solves of a mixed-form sub-step interleaved on two
// streams. The FP64 defects (FP64-pipe bound, on the persistent grid) stay on
// the solver's stream; as soon as a component's defect norm reaches the host
// and asks for a correction, that correction (Gauss-Seidel sweeps on e32 from
// d32c[c], then x += e) goes to the auxiliary stream, where it runs beside
// the next component's defect, and the component's next defect is queued
// behind it. Components are served in the order their defects were queued.
// Each component goes through exactly the steps of helm_solve_mixed (same
// defects, corrections and stopping test, bit for bit); only the order of
// the norms' partial sums differs. first(c) launches component c's first
// defect into d32c[c] with its squared norm in scal[12 + c]. Needs the
// Gauss-Seidel inner solve (helm_overlap_ok). With per-kernel profiling on,
// each launch is timed by events on its own stream (durations of kernels
// that ran side by side overlap).
bool helm_overlap_ok(afmib_solver* s, double scale) {
    const Dims& d = s->d;
    return s->helm_overlap && s->aux && s->hi && s->gs_inner && !s->bfp_defects &&
           gs_sweeps(d, scale, s->cfg.inner_tol) > 0 && d.nz % 8 == 0 && d.nx % 2 == 0 && ix2_ok(d);
}

template <typename F>
int helm_solve3_mixed(afmib_solver* s, double scale, double* const x[3], const double* const b[3], F first) {
    const Dims& d = s->d;
    const long long N = s->N();
    const int gsw = gs_sweeps(d, scale, s->cfg.inner_tol);
    const bool big = s->alternate && (double)N * sizeof(float) >= 32.0 * (1 << 20);
    cudaStream_t hs = s->hi;
    const bool df = s->helm_df && s->rlo[0];
    auto post = [&](int c, cudaStream_t q) -> int {
        CK(cudaMemcpyAsync(s->hscal + 12 + c, s->scal + 12 + c, sizeof(double), cudaMemcpyDeviceToHost, q));
        CK(cudaEventRecord(s->ev_def[c], q));
        return AFMIB_OK;
    };
    CK(cudaEventRecord(s->ev_join, s->st));
    CK(cudaStreamWaitEvent(hs, s->ev_join, 0));
    int ring[3], head = 0, count = 0, outer[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) {
        first(c, hs, df ? s->rlo[c] : nullptr);
        CKL();
        TRY(post(c, hs));
        ring[count++] = c;
    }
    int status = AFMIB_OK;
    while (count > 0) {
        const int c = ring[head];
        head = (head + 1) % 3;
        --count;
        CK(cudaEventSynchronize(s->ev_def[c]));
        const double nr = std::sqrt(s->hscal[12 + c]);
        s->stats.last_cg_norm = nr;
        if (!std::isfinite(nr)) { status = s->fail(AFMIB_ERR_NAN, "Helmholtz residual is not finite"); break; }
        if (nr <= s->cfg.tol) {
            s->stats.outer_iters += outer[c];
            continue;
        }
        if (outer[c] >= s->cfg.max_mg_cycles) {
            status = s->fail(AFMIB_ERR_NOCONV, "defect-correction cap reached (Helmholtz)");
            break;
        }
        CK(cudaStreamWaitEvent(s->aux, s->ev_def[c], 0));
        int rev = 1;  // the defect's walk ended at the last z planes
        for (int j = 0; j < gsw; ++j)
            for (int color = 0; color < 2; ++color) {
                ProfScope ps(s, P_JACOBI, (double)N * 4 * 1.5, 1, s->aux);
                launch_helm_rbgs<float>(d, c, scale, color, j == 0 && color == 0, s->e32, s->d32c[c], s->aux,
                                        big ? rev : 0);
                rev ^= 1;
            }
        if (df) {
            ProfScope ps(s, P_HELM_UPDATE, (double)N * (8 + 4 + 8 + 8 + 8 + 4), 1, s->aux);
            launch_helm_update_df(d, c, scale, x[c], s->e32, s->d32c[c], s->rlo[c], s->red2, s->scal + 12 + c,
                                  s->aux);
            CKL();
            TRY(post(c, s->aux));
            ring[(head + count++) % 3] = c;
            ++outer[c];
            continue;
        }
        {
            ProfScope ps(s, P_CORRECT, (double)N * (8 + 4 + 8), 1, s->aux);
            launch_add_correction<float>(N, x[c], s->e32, s->aux);
        }
        CKL();
        CK(cudaEventRecord(s->ev_cor[c], s->aux));
        CK(cudaStreamWaitEvent(hs, s->ev_cor[c], 0));
        {
            ProfScope ps(s, P_HELM_DEFECT, (double)N * (8 + 8 + 4), 1, hs);
            launch_helm_defect<float>(d, c, scale, x[c], b[c], s->d32c[c], s->red, s->scal + 12 + c, hs,
                                      s->walk_blocks);
        }
        CKL();
        TRY(post(c, hs));
        ring[(head + count++) % 3] = c;
        ++outer[c];
    }
    if (status != AFMIB_OK) {
        cudaStreamSynchronize(s->aux);
        cudaStreamSynchronize(hs);
        cudaStreamSynchronize(s->st);
        return status;
    }
    // FP64 defects: every correction was followed by a defect on hs, so
    // joining hs joins both; double-float updates: join both streams
    CK(cudaEventRecord(s->ev_join, hs));
    CK(cudaStreamWaitEvent(s->st, s->ev_join, 0));
    if (df) {
        CK(cudaEventRecord(s->ev_cor[0], s->aux));
        CK(cudaStreamWaitEvent(s->st, s->ev_cor[0], 0));
    }
    return AFMIB_OK;
}

int mg_solve_mixed(afmib_solver* s, int* cycles) {
    MGLevel& L = s->lv[0];
    MGLevelT<float>& L32 = s->lv32[0];
    const long long N = L.d.ncell();
    const double Ns = (double)N * sizeof(double);
    const bool df = lap_df_on(s);
    // double-float first defect: b's mean is subtracted inside it (b is read
    // by the first defect only; the later ones are the recursive updates)
    const bool fuse_mean = df && s->proj_df;
    if (!s->b_sum_ready || !fuse_mean) {
        ProfScope ps(s, P_MEAN, (s->b_sum_ready ? 0 : Ns) + (fuse_mean ? 0 : 2 * Ns),
                     (s->b_sum_ready ? 0 : 1) + (fuse_mean ? 0 : 1));
        if (!s->b_sum_ready) launch_sum<double>(N, L.b, s->red, s->scal + 8, s->st);
        if (!fuse_mean) launch_sub_scalar_scaled<double>(N, L.b, s->scal + 8, 1.0 / (double)N, s->st);
    }
    s->b_sum_ready = false;
    TRY(initial_potential(s));
    CK(cudaMemsetAsync(s->dflag + 1, 0, sizeof(int), s->st));
    int c = 0, outer = 0, last_cyc = 0;
    double last_rms = 0.0;
    int status = AFMIB_OK;
    for (;;) {
        if (!(df && outer > 0)) {  // double-float: the norm came with the last block's update
            ProfScope ps(s, P_LAP_DEFECT, (double)N * (8 + 8 + 4 + (df ? 4 : 0)));
            if (fuse_mean)
                launch_lap_defect_df(L.d, L32.b, s->plo, L.x, L.b, s->scal + 8, 1.0 / (double)N, s->red, s->scal + 9,
                                     s->st);
            else if (!s->bfp_defects || !launch_lap_defect_bfp(L.d, L32.b, L.x, L.b, s->red, s->scal + 9, s->st))
                launch_lap_defect<float>(L.d, L32.b, L.x, L.b, s->red, s->scal + 9, s->st, df ? s->plo : nullptr);
        }
        CKL();
        TRY(read_scalars(s, 9, 1));
        const double rms = std::sqrt(s->hscal[9]) / std::sqrt((double)N);
        s->stats.last_mg_rms = rms;
        if (!std::isfinite(rms)) { status = s->fail(AFMIB_ERR_NAN, "multigrid residual is not finite"); break; }
        if (last_cyc > 0 && rms > 0.0 && rms < last_rms) s->mg_rho = std::pow(rms / last_rms, 1.0 / last_cyc);
        if (rms <= s->cfg.tol) break;
        if (c >= s->cfg.max_mg_cycles) { status = s->fail(AFMIB_ERR_NOCONV, "multigrid cycle cap reached"); break; }
        int cyc = s->inner_cycles;
        if (s->adapt_cycles && s->mg_rho > 0.0) {
            const double need = std::log(0.5 * s->cfg.tol / rms) / std::log(s->mg_rho);
            if (need < cyc) cyc = std::max(1, (int)std::ceil(need));
        }
        TRY(inner_vcycles32(s, cyc));
        c += cyc;
        ++outer;
        last_rms = rms;
        last_cyc = cyc;
    }
    CK(cudaMemcpyAsync(s->hflag + 1, s->dflag + 1, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(s->hflag + 3, s->dflag + 3, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    TRY(sync(s));
    if (s->hflag[3] != 0) return s->fail(AFMIB_ERR_CUDA, "pipelined smoother: a row copy did not complete in time");
    if (status == AFMIB_OK && s->hflag[1] != 0) status = s->fail(AFMIB_ERR_NOCONV, "coarsest-level CG did not converge");
    s->stats.mg_cycles += c;
    s->stats.outer_iters += outer;
    if (cycles) *cycles = c;
    return status;
}

// ns::projection::project, src/ns/projection.h:60-73
int project(afmib_solver* s) {
    const double Ns = (double)s->N() * sizeof(double);
    const bool pdf = s->mixed && s->proj_df;
    s->b_sum_ready = false;
    {
        ProfScope ps(s, P_DIV, 4 * Ns);
        if (pdf) {
            launch_div_df(s->d, s->lv[0].b, s->u, s->v, s->w, nullptr, nullptr, s->red, s->scal + 8, s->st);
            s->b_sum_ready = true;
        } else {
            launch_div<double>(s->d, s->lv[0].b, s->u, s->v, s->w, nullptr, nullptr, s->st);
        }
    }
    CKL();
    if (s->mixed) TRY(mg_solve_mixed(s, nullptr));
    else TRY(mg_solve(s, nullptr));
    const int ph = s->proj_phase;
    if (s->warm_start && ph >= 0) {
        if (s->warm_extrap) {
            std::swap(s->phi_prev[ph], s->phi_prev2[ph]);
            s->phi_valid2[ph] = s->phi_valid[ph];
        }
        CK(cudaMemcpyAsync(s->phi_prev[ph], s->lv[0].x, s->N() * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        s->phi_valid[ph] = true;
    }
    {
        ProfScope ps(s, P_GRAD_SUB, 7 * Ns);
        launch_grad_sub<double>(s->d, s->u, s->v, s->w, s->lv[0].x, s->d.channel ? s->wallgrad : nullptr, s->st,
                                s->u32, s->v32, s->w32, s->round_shadow, s->u32l, s->v32l, s->w32l);
    }
    CKL();
    return AFMIB_OK;
}

// ns::solver::step, src/ns/solver.h:90-140; forces already in s->f (FP64
// form) or s->f32 (mixed form).
int substep(afmib_solver* s) {
    const Dims& d = s->d;
    const long long N = s->N();
    const double Ns = (double)N * sizeof(double);
    if (s->mixed && s->advect64) {
        // FP64 advection of the FP64 velocity, handed on in FP32
        ProfScope ps(s, P_ADVECT, 6 * Ns + (double)N * 3 * 4, 4);
        launch_advect<double, double>(d, s->adv[0], s->adv[1], s->adv[2], s->u, s->v, s->w, s->st);
        for (int k = 0; k < 3; ++k) launch_convert<float, double>(N, s->adv32[k], s->adv[k], s->st);
    } else if (s->mixed && s->u32l) {
        ProfScope ps(s, P_ADVECT, (double)N * (6 * 4 + 3 * 4));
        launch_advect_df(d, s->adv32[0], s->adv32[1], s->adv32[2], s->u32, s->u32l, s->v32, s->v32l, s->w32, s->w32l,
                         s->st);
    } else if (s->mixed) {
        ProfScope ps(s, P_ADVECT, (double)N * (3 * 4 + 3 * 4));
        launch_advect<float, float>(d, s->adv32[0], s->adv32[1], s->adv32[2], s->u32, s->v32, s->w32, s->st);
    } else {
        ProfScope ps(s, P_ADVECT, 6 * Ns);
        launch_advect<double, double>(d, s->adv[0], s->adv[1], s->adv[2], s->u, s->v, s->w, s->st);
    }
    CKL();
    const bool be = !s->half;
    // the fused mixed-form path copies u into uo inside its first pass
    const bool fused = s->mixed && s->fused_rhs && s->qo[0] && !s->bfp_defects;
    if (be && !fused) {
        CK(cudaMemcpyAsync(s->uo[0], s->u, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(s->uo[1], s->v, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(s->uo[2], s->w, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    }
    if (d.channel) {
        ProfScope ps(s, P_WALL, 10.0 * s->nxz() * sizeof(double));
        launch_wall_update(d, s->walls, s->wallgrad, s->st, s->cfg.walls_corrected);
    }
    const long long nxz = s->nxz();
    const double* ut = s->walls;
    const double* ub = s->walls + nxz;
    const double* wt = s->walls + 2 * nxz;
    const double* wb = s->walls + 3 * nxz;
    const double inv_rho = 1 / s->cfg.rho;
    double* vel[3] = {s->u, s->v, s->w};
    if (fused) {
        // backward Euler: right-hand side, first defect (x starts at uold),
        // Q(uold) and the copy of uold in one pass per component;
        // Crank-Nicolson: right-hand sides from Q(uold), then the solves
        const bool ovl = helm_overlap_ok(s, s->s_minus());
        auto walls_of = [&](int c, const double** top, const double** bot) {
            *top = (!d.channel || c == 1) ? nullptr : (c == 0 ? ut : wt);
            *bot = (!d.channel || c == 1) ? nullptr : (c == 0 ? ub : wb);
        };
        auto be_first = [&](int c, float* r, double* out, int wblocks, cudaStream_t q, float* lo) {
            const double *top, *bot;
            walls_of(c, &top, &bot);
            ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 8 + 4 + 8 + 8 + 4), 1, q);
            if (s->spread64 && lo && s->first_df)
                launch_helm_rhs_be_defect_df<float>(d, c, r, lo, s->qo[c], s->uo[c], vel[c], s->f[c], s->adv32[c], top,
                                                    bot, s->s_minus(), s->cfg.dt, inv_rho, s->red, out, q, wblocks);
            else if (s->spread64)
                launch_helm_rhs_be_defect<double, float>(d, c, s->rhs[c], r, s->qo[c], vel[c], s->f[c], s->adv32[c],
                                                         top, bot, s->s_minus(), s->cfg.dt, inv_rho, s->red, out, q,
                                                         wblocks, lo, s->uo[c]);
            else
                launch_helm_rhs_be_defect<float, float>(d, c, s->rhs[c], r, s->qo[c], vel[c], s->f32[c],
                                                        s->adv32[c], top, bot, s->s_minus(), s->cfg.dt, inv_rho,
                                                        s->red, out, q, wblocks, lo, s->uo[c]);
        };
        if (be) {
            if (ovl) {
                TRY(helm_solve3_mixed(s, s->s_minus(), vel, s->rhs, [&](int c, cudaStream_t hs, float* lo) {
                    be_first(c, s->d32c[c], s->scal + 12 + c, s->walk_blocks_be, hs, lo);
                }));
            } else {
                for (int c = 0; c < 3; ++c) {
                    be_first(c, s->d32, s->scal + 10, 0, s->st, nullptr);
                    CKL();
                    TRY(helm_solve_mixed(s, c, s->s_minus(), vel[c], s->rhs[c], true));
                }
            }
            s->qo_valid = true;
        } else {
            const bool cn_first = ovl && s->helm_df && s->rlo[0] && s->qo_valid && s->cn_start_old;
            for (int c = 0; c < 3 && !cn_first; ++c) {
                const double *top, *bot;
                walls_of(c, &top, &bot);
                if (s->qo_valid) {
                    ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 8 + 8 + 4 + 8));
                    if (s->spread64)
                        launch_helm_rhs_cn_q<double, float>(d, c, s->rhs[c], s->uo[c], s->qo[c], s->f[c], s->adv32[c],
                                                            top, bot, s->s_plus(), s->s_minus(), s->cfg.dt, inv_rho,
                                                            s->st);
                    else
                        launch_helm_rhs_cn_q<float, float>(d, c, s->rhs[c], s->uo[c], s->qo[c], s->f32[c],
                                                           s->adv32[c], top, bot, s->s_plus(), s->s_minus(),
                                                           s->cfg.dt, inv_rho, s->st);
                } else if (s->spread64) {
                    ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 8 + 4 + 8));
                    launch_helm_rhs<double, double, float>(d, c, 0, s->rhs[c], s->uo[c], s->f[c], s->adv32[c], top,
                                                           bot, s->s_plus(), s->s_minus(), s->cfg.dt, inv_rho, s->st);
                } else {
                    ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 4 + 4 + 8));
                    launch_helm_rhs<double, float, float>(d, c, 0, s->rhs[c], s->uo[c], s->f32[c], s->adv32[c], top,
                                                          bot, s->s_plus(), s->s_minus(), s->cfg.dt, inv_rho, s->st);
                }
            }
            CKL();
            if (ovl) {
                TRY(helm_solve3_mixed(s, s->s_minus(), vel, s->rhs, [&](int c, cudaStream_t hs, float* lo) {
                    if (cn_first) {
                        const double *top, *bot;
                        walls_of(c, &top, &bot);
                        ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 8 + 8 + 4 + 8 + 4 + 4), 1, hs);
                        if (s->spread64 && s->first_df)
                            launch_helm_cn_first_df<float>(d, c, vel[c], s->d32c[c], lo, s->uo[c], s->qo[c], s->f[c],
                                                           s->adv32[c], top, bot, s->s_plus(), s->s_minus(),
                                                           s->cfg.dt, inv_rho, s->red, s->scal + 12 + c, hs);
                        else if (s->spread64)
                            launch_helm_cn_first<double, float>(d, c, vel[c], s->d32c[c], lo, s->uo[c], s->qo[c],
                                                                s->f[c], s->adv32[c], top, bot, s->s_plus(),
                                                                s->s_minus(), s->cfg.dt, inv_rho, s->red,
                                                                s->scal + 12 + c, hs);
                        else
                            launch_helm_cn_first<float, float>(d, c, vel[c], s->d32c[c], lo, s->uo[c], s->qo[c],
                                                               s->f32[c], s->adv32[c], top, bot, s->s_plus(),
                                                               s->s_minus(), s->cfg.dt, inv_rho, s->red,
                                                               s->scal + 12 + c, hs);
                        return;
                    }
                    ProfScope ps(s, P_HELM_DEFECT, (double)N * (8 + 8 + 4), 1, hs);
                    launch_helm_defect<float>(d, c, s->s_minus(), vel[c], s->rhs[c], s->d32c[c], s->red,
                                              s->scal + 12 + c, hs, s->walk_blocks, lo);
                }));
            } else {
                for (int c = 0; c < 3; ++c) TRY(helm_solve_mixed(s, c, s->s_minus(), vel[c], s->rhs[c]));
            }
        }
        s->proj_phase = be ? 0 : 1;
        const int prc = project(s);
        s->proj_phase = -1;
        TRY(prc);
        s->half = !s->half;
        s->stats.half = s->half ? 1 : 0;
        s->stats.substeps++;
        return AFMIB_OK;
    }
    for (int c = 0; c < 3; ++c) {
        const double* top = (!d.channel || c == 1) ? nullptr : (c == 0 ? ut : wt);
        const double* bot = (!d.channel || c == 1) ? nullptr : (c == 0 ? ub : wb);
        if (s->mixed && s->spread64) {
            ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 8 + 4 + 8));
            launch_helm_rhs<double, double, float>(d, c, be ? 1 : 0, s->rhs[c], s->uo[c], s->f[c], s->adv32[c], top,
                                                   bot, s->s_plus(), s->s_minus(), s->cfg.dt, inv_rho, s->st);
        } else if (s->mixed) {
            ProfScope ps(s, P_HELM_RHS, (double)N * (8 + 4 + 4 + 8));
            launch_helm_rhs<double, float, float>(d, c, be ? 1 : 0, s->rhs[c], s->uo[c], s->f32[c], s->adv32[c], top,
                                                  bot, s->s_plus(), s->s_minus(), s->cfg.dt, inv_rho, s->st);
        } else {
            ProfScope ps(s, P_HELM_RHS, 4 * Ns);
            launch_helm_rhs<double, double, double>(d, c, be ? 1 : 0, s->rhs[c], s->uo[c], s->f[c], s->adv[c], top, bot,
                                            s->s_plus(), s->s_minus(), s->cfg.dt, inv_rho, s->st);
        }
    }
    CKL();
    for (int c = 0; c < 3; ++c) {
        if (s->mixed) TRY(helm_solve_mixed(s, c, s->s_minus(), vel[c], s->rhs[c]));
        else TRY(cg_solve(s, c, s->s_minus(), vel[c], s->rhs[c], nullptr));
    }
    s->proj_phase = be ? 0 : 1;
    const int prc = project(s);
    s->proj_phase = -1;
    TRY(prc);
    s->half = !s->half;
    s->stats.half = s->half ? 1 : 0;
    s->stats.substeps++;
    return AFMIB_OK;
}

// ---------------------------------------------------------------------------
// Immersed boundary
// ---------------------------------------------------------------------------
// (re)allocate a device buffer, keeping the first `keep` elements
template <typename T>
int regrow(afmib_solver* s, T** p, size_t count, size_t keep) {
    T* q = nullptr;
    TRY(dalloc(s, &q, count));
    if (*p) {
        if (keep) CK(cudaMemcpyAsync(q, *p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaStreamSynchronize(s->st));
        for (auto& a : s->allocs)
            if (a == (void*)*p) { cudaFree(a); a = nullptr; }
    }
    *p = q;
    return AFMIB_OK;
}

// Grow the marker buffers to M markers and nnz neighbour entries. The
// solver's own marker set (X, nstart, nidx, vol) survives a growth; the
// other buffers are per-call workspace.
int marker_alloc(afmib_solver* s, int M, int nnz) {
    if (M > s->Mcap) {
        const size_t keep = (size_t)s->M;
        TRY(regrow(s, &s->X, 3 * (size_t)M, 3 * keep));
        TRY(regrow(s, &s->nstart, (size_t)M + 1, keep ? keep + 1 : 0));
        TRY(regrow(s, &s->mvol, (size_t)M, keep));
        TRY(regrow(s, &s->Xh, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->Ybend, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->U1, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->U2, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->G, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->keys, (size_t)M, 0));
        TRY(regrow(s, &s->keys2, (size_t)M, 0));
        TRY(regrow(s, &s->vals, (size_t)M, 0));
        TRY(regrow(s, &s->vals2, (size_t)M, 0));
        TRY(regrow(s, &s->hist, radix_sort_temp_bytes(M) / sizeof(unsigned) + 256, 0));
        TRY(regrow(s, &s->mw.cell, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->mw.dbase, 6 * (size_t)M, 0));
        TRY(regrow(s, &s->mw.w, 24 * (size_t)M, 0));
        TRY(regrow(s, &s->mw32.cell, 3 * (size_t)M, 0));
        TRY(regrow(s, &s->mw32.dbase, 6 * (size_t)M, 0));
        TRY(regrow(s, &s->mw32.w, 24 * (size_t)M, 0));
        TRY(regrow(s, &s->G32, 3 * (size_t)M, 0));
        s->Mcap = M;
    }
    {
        const int need = std::min(s->ntiles, std::max(M, 1));
        if (need > s->ctab_cap) {
            TRY(regrow(s, &s->ctab, (size_t)need * (s->tile_cells() + 1), 0));
            s->ctab_cap = need;
        }
    }
    if (nnz > s->nnz_cap) {
        TRY(regrow(s, &s->nidx, (size_t)nnz, 0));
        s->nnz_cap = nnz;
    }
    return AFMIB_OK;
}

int key_bits(afmib_solver* s) {
    const unsigned long long top = (unsigned long long)s->ntiles * s->tile_cells();
    int b = 0;
    while ((1ull << b) < top) ++b;
    return b;
}

// weights + bins of the markers at P (device, [M][3])
// df_weights: the FP64 weights by launch_marker_prep's double-float sine and
// cosine (the mixed form's IB step)
int bin_markers(afmib_solver* s, const double* P, bool fp32 = false, bool df_weights = false) {
    const int M = s->M;
    const int passes = (key_bits(s) + 7) / 8;
    if (fp32) {
        ProfScope ps(s, P_PREP, (double)M * (24 + 4 + 4 + 12 + 6 + 24 * 4));
        launch_marker_prep<float>(s->d, s->TS, M, P, s->keys, s->vals, s->mw32, s->dflag, s->st);
    } else {
        ProfScope ps(s, P_PREP, (double)M * (24 + 4 + 4 + 12 + 6 + 24 * 8));
        launch_marker_prep<double>(s->d, s->TS, M, P, s->keys, s->vals, s->mw, s->dflag, s->st, df_weights);
    }
    unsigned* ko;
    int* vo;
    {
        ProfScope ps(s, P_SORT, (double)passes * M * 16, 3 * passes);
        radix_sort_pairs(s->keys, s->vals, s->keys2, s->vals2, M, key_bits(s), s->hist, &ko, &vo, s->st);
    }
    s->perm = vo;
    CK(cudaMemsetAsync(s->tstart, 0, s->ntiles * sizeof(int), s->st));
    CK(cudaMemsetAsync(s->tend, 0, s->ntiles * sizeof(int), s->st));
    CK(cudaMemsetAsync(s->tcount, 0, 2 * sizeof(int), s->st));
    {
        const int C = s->tile_cells();
        ProfScope ps(s, P_TILES, (double)M * 4 + 5.0 * s->ntiles * 4 + (double)std::min(M, s->ntiles) * (C + 1) * 4, 3);
        launch_tile_ranges(ko, M, C, s->tstart, s->tend, s->st);
        launch_active_tiles(s->ntx, s->nty, s->ntz, s->d.channel, s->tstart, s->tend, s->tlist, s->tcount, s->tslot,
                            s->tocc, s->tcount + 1, s->st);
        launch_cell_table(s->TS, s->TZ, ko, s->tstart, s->tend, s->tocc, s->tcount + 1, s->ctab_cap, s->ctab, s->st);
    }
    CKL();
    return AFMIB_OK;
}

// Spreading in two passes: blocks sized for `cap_small` neighbourhood markers
// (two blocks per SM) take every active tile whose neighbourhood fits and list
// the others, which a second pass with `cap_large` handles. Each tile is
// computed once, by one of the passes, with the same arithmetic.
template <typename T>
int spread_two_pass(afmib_solver* s, MarkerW<T> mw, const T* G, const double* vol, double scale, T* fu, T* fv, T* fw,
                    int cap_small, int cap_large, bool dfloat = false) {
    CK(cudaMemsetAsync(s->tcount + 2, 0, 3 * sizeof(int), s->st));  // overflow count and the two tile counters
    launch_spread_gather<T>(s->d, s->TS, s->M, s->perm, mw, G, vol, scale, s->tslot, s->ctab, s->tlist, s->tcount,
                            s->ntiles, cap_small, fu, fv, fw, s->tovf, s->tcount + 2, s->tcount + 3, s->st, dfloat);
    launch_spread_gather<T>(s->d, s->TS, s->M, s->perm, mw, G, vol, scale, s->tslot, s->ctab, s->tovf, s->tcount + 2,
                            s->ntiles, cap_large, fu, fv, fw, nullptr, nullptr, s->tcount + 4, s->st, dfloat);
    return AFMIB_OK;
}

// f = scale * S(X) G with the FP64 bins and weights of the last bin_markers call
int spread_generic(afmib_solver* s, const double* G, const double* vol, double scale, double* fu, double* fv,
                   double* fw) {
    const long long N = s->N();
    CK(cudaMemsetAsync(fu, 0, N * sizeof(double), s->st));
    CK(cudaMemsetAsync(fv, 0, N * sizeof(double), s->st));
    CK(cudaMemsetAsync(fw, 0, N * sizeof(double), s->st));
    const double touched = (double)s->stats.spread_tiles * s->tile_cells();
    {
        ProfScope ps(s, P_SPREAD, (double)s->M * (24 + 3 * 8 + 8 + 8) + 3 * touched * 8);
        TRY(spread_two_pass<double>(s, s->mw, G, vol, scale, fu, fv, fw, 896, 1536));
    }
    CKL();
    return AFMIB_OK;
}

// Spreading scale phi^3 / (phi/n)^3 = n^3; on a 2D grid the kernel is
// phi^2 = n^2 (phi/n)^2 (a marker's volume is then its area measure).
double spread_scale(const Dims& d) {
    return d.nz == 1 ? (double)d.n * d.n : (double)d.n * d.n * d.n;
}

// f = spread(G) with the bins and weights of the last bin_markers call.
// Algorithmic bytes: M (24 + 3s + 8 + 8) + 3 N_touched s with N_touched
// taken as the faces of the active tiles (from the previous spreading).
int spread_forces(afmib_solver* s, const double* vol, double* fu, double* fv, double* fw, bool dfloat = false) {
    const long long N = s->N();
    CK(cudaMemsetAsync(fu, 0, N * sizeof(double), s->st));
    CK(cudaMemsetAsync(fv, 0, N * sizeof(double), s->st));
    CK(cudaMemsetAsync(fw, 0, N * sizeof(double), s->st));
    const double n3 = spread_scale(s->d);
    const int cap = 1536;
    const double touched = (double)s->stats.spread_tiles * s->tile_cells();
    {
        ProfScope ps(s, P_SPREAD, (double)s->M * (24 + 3 * 8 + 8 + 8) + 3 * touched * 8);
        TRY(spread_two_pass<double>(s, s->mw, s->G, vol, n3, fu, fv, fw, 896, cap, dfloat));
    }
    CKL();
    return AFMIB_OK;
}

int spread_forces32(afmib_solver* s, const double* vol) {
    const long long N = s->N();
    for (int c = 0; c < 3; ++c) CK(cudaMemsetAsync(s->f32[c], 0, N * sizeof(float), s->st));
    const double n3 = spread_scale(s->d);
    const int cap = 3072;
    const double touched = (double)s->stats.spread_tiles * s->tile_cells();
    {
        ProfScope ps(s, P_SPREAD, (double)s->M * (24 + 3 * 4 + 8 + 8) + 3 * touched * 4);
        TRY(spread_two_pass<float>(s, s->mw32, s->G32, vol, n3, s->f32[0], s->f32[1], s->f32[2], 1792, cap));
    }
    CKL();
    return AFMIB_OK;
}

int check_marker_flag(afmib_solver* s) {
    CK(cudaMemcpyAsync(s->hflag, s->dflag, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(s->hflag + 2, s->tcount, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    TRY(sync(s));
    s->stats.spread_tiles = s->hflag[2];
    const int f = s->hflag[0];
    if (f == 1) return s->fail(AFMIB_ERR_BOUNDS, "a marker came within 2.5h of a channel wall");
    if (f == 2) return s->fail(AFMIB_ERR_NAN, "a marker position is not finite");
    return AFMIB_OK;
}

// pairs: u, v, w are the solver's velocity and its float pairs (u32 +
// u32l, ...) are current (after a projection or a velocity set)
int interp_markers(afmib_solver* s, const double* u, const double* v, const double* w, double* U, bool fp32 = false,
                   bool dfloat = false, bool pairs = false) {
    const double touched = (double)s->stats.spread_tiles * s->tile_cells();
    ProfScope ps(s, P_INTERP, 3 * touched * 8 + (double)s->M * (24 + 3 * 8 + 8));
    if (fp32) launch_interp<float, float>(s->d, s->M, s->perm, s->mw32, s->u32, s->v32, s->w32, U, s->st);
    else if (dfloat && pairs && s->interp_pairs && s->u32 && s->u32l)
        launch_interp_dfl(s->d, s->M, s->perm, s->mw, u, v, w, U, s->st, s->u32, s->u32l, s->v32, s->v32l, s->w32,
                          s->w32l);
    else if (dfloat) launch_interp_dfl(s->d, s->M, s->perm, s->mw, u, v, w, U, s->st);
    else launch_interp<double, double>(s->d, s->M, s->perm, s->mw, u, v, w, U, s->st);
    return AFMIB_OK;
}

int ib_one_step(afmib_solver* s) {
    const int M = s->M;
    const double dt = s->cfg.dt;
    const double* vol = s->has_vol ? s->mvol : nullptr;
    const double mbytes = (double)M * (24 + 24 + 24);
    // precision of each transfer: FP64 form -> FP64; mixed -> FP64 unless ib_fp32 asks for FP32
    const bool sp32 = s->mixed && !s->spread64;
    const bool in32 = s->mixed && !s->interp64;
    auto springs = [&](const double* P) {
        ProfScope ps(s, P_SPRINGS, mbytes);
        const double ks = s->cfg.k_spring, kb = s->cfg.k_bend;
        if (kb != 0.0) {
            if (sp32) launch_springs_bending<float>(M, P, s->nstart, s->nidx, ks, kb, s->Ybend, s->G32, s->st);
            else launch_springs_bending<double>(M, P, s->nstart, s->nidx, ks, kb, s->Ybend, s->G, s->st);
        } else if (sp32) {
            launch_springs<float>(M, P, s->nstart, s->nidx, ks, s->G32, s->st);
        } else {
            launch_springs<double>(M, P, s->nstart, s->nidx, ks, s->G, s->st);
        }
    };
    // the mixed form's FP64 weights from double-float sines and cosines
    const bool dfw = s->mixed && s->prep_df;
    auto bin = [&](const double* P) -> int {
        TRY(bin_markers(s, P, sp32, dfw));
        if (sp32 != in32) {  // the other weight set for the other transfer (same bins)
            ProfScope ps(s, P_PREP, (double)M * (24 + 4 + 4 + 12 + 6 + 24 * (in32 ? 4 : 8)));
            if (in32) launch_marker_prep<float>(s->d, s->TS, M, P, nullptr, nullptr, s->mw32, s->dflag, s->st);
            else launch_marker_prep<double>(s->d, s->TS, M, P, nullptr, nullptr, s->mw, s->dflag, s->st, dfw);
        }
        return AFMIB_OK;
    };
    auto spread = [&]() {
        return sp32 ? spread_forces32(s, vol)
                    : spread_forces(s, vol, s->f[0], s->f[1], s->f[2], s->mixed && s->spread_df);
    };
    auto interp = [&](double* U) {
        return in32 ? interp_markers(s, s->u, s->v, s->w, U, true)
                    : interp_markers(s, s->u, s->v, s->w, U, false, s->mixed && s->interp_df, true);
    };
    CK(cudaMemsetAsync(s->dflag, 0, sizeof(int), s->st));
    const long long N = s->N();
    if (s->recording) {
        double* r = s->rec_u0[s->rec_j];
        CK(cudaMemcpyAsync(r, s->u, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(r + N, s->v, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(r + 2 * N, s->w, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(s->rec_X0[s->rec_j], s->X, 3 * (size_t)M * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    }
    // BE half: forces at X^n
    springs(s->X);
    TRY(bin(s->X));
    TRY(spread());
    TRY(substep(s));
    if (s->recording) {
        double* r = s->rec_uh[s->rec_j];
        CK(cudaMemcpyAsync(r, s->u, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(r + N, s->v, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
        CK(cudaMemcpyAsync(r + 2 * N, s->w, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    }
    // velocity at t+dt/2: at X^n for the half-step, then at X^{n+1/2}
    TRY(interp(s->U1));
    {
        ProfScope ps(s, P_MARKER, mbytes);
        launch_marker_axpy(M, s->Xh, s->X, s->U1, dt / 2, s->st);
    }
    if (s->recording)
        CK(cudaMemcpyAsync(s->rec_Xh[s->rec_j], s->Xh, 3 * (size_t)M * sizeof(double), cudaMemcpyDeviceToDevice,
                           s->st));
    TRY(bin(s->Xh));
    TRY(interp(s->U2));
    // CN step with forces at X^{n+1/2}
    springs(s->Xh);
    CKL();
    TRY(spread());
    TRY(substep(s));
    {
        ProfScope ps(s, P_MARKER, mbytes);
        launch_marker_axpy(M, s->X, s->X, s->U2, dt, s->st);
    }
    CKL();
    TRY(check_marker_flag(s));
    s->stats.ib_steps++;
    return AFMIB_OK;
}

// ---------------------------------------------------------------------------
// Trajectory and adjoint. The forward trajectory stores the state (u, X) every
// `every` steps; the reverse pass recomputes one segment at a time from its
// checkpoint, recording u^n, u^{n+1/2}, X^n and X^{n+1/2} of each step, and
// runs the reverse IB step over the records (periodic domain). In the
// periodic domain the projection P and the Helmholtz operator H = I - s Delta
// are symmetric, so their adjoints reuse the forward multigrid and CG solves.
// ---------------------------------------------------------------------------
int copy_vel_out(afmib_solver* s, double* dst) {
    const long long N = s->N();
    CK(cudaMemcpyAsync(dst, s->u, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    CK(cudaMemcpyAsync(dst + N, s->v, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    CK(cudaMemcpyAsync(dst + 2 * N, s->w, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    return AFMIB_OK;
}

int refresh_shadow(afmib_solver* s);

int copy_vel_in(afmib_solver* s, const double* src) {
    const long long N = s->N();
    CK(cudaMemcpyAsync(s->u, src, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    CK(cudaMemcpyAsync(s->v, src + N, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    CK(cudaMemcpyAsync(s->w, src + 2 * N, N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    return refresh_shadow(s);
}

// (u, v, w) <- P (u, v, w)
int project_fields(afmib_solver* s, double* u, double* v, double* w) {
    launch_div<double>(s->d, s->lv[0].b, u, v, w, nullptr, nullptr, s->st);
    CKL();
    if (s->mixed) TRY(mg_solve_mixed(s, nullptr));
    else TRY(mg_solve(s, nullptr));
    launch_grad_sub<double>(s->d, u, v, w, s->lv[0].x, nullptr, s->st);
    CKL();
    return AFMIB_OK;
}

// x <- H^{-1} b for each component, from a zero start
int helm_inverse(afmib_solver* s, double* x, const double* b) {
    const long long N = s->N();
    CK(cudaMemsetAsync(x, 0, 3 * N * sizeof(double), s->st));
    for (int c = 0; c < 3; ++c) {
        if (s->mixed) TRY(helm_solve_mixed(s, c, s->s_minus(), x + c * N, b + c * N));
        else TRY(cg_solve(s, c, s->s_minus(), x + c * N, b + c * N, nullptr));
    }
    return AFMIB_OK;
}

int traj_alloc(afmib_solver* s, int nsteps, int every) {
    const long long N = s->N();
    const int M = s->M;
    const int nck = (nsteps + every - 1) / every;
    auto grow = [&](std::vector<double*>& v, int count, size_t len) -> int {
        while ((int)v.size() < count) {
            double* p = nullptr;
            TRY(dalloc(s, &p, len));
            v.push_back(p);
        }
        return AFMIB_OK;
    };
    if (s->traj_M != M) {  // marker count changed: drop marker-sized buffers
        s->ck_X.clear(); s->rec_X0.clear(); s->rec_Xh.clear();
        s->fin_X = nullptr; s->lamX = nullptr;
        s->traj_M = M;
    }
    TRY(grow(s->ck_vel, nck, 3 * N));
    TRY(grow(s->ck_X, nck, 3 * (size_t)M));
    TRY(grow(s->rec_u0, every, 3 * N));
    TRY(grow(s->rec_uh, every, 3 * N));
    TRY(grow(s->rec_X0, every, 3 * (size_t)M));
    TRY(grow(s->rec_Xh, every, 3 * (size_t)M));
    if (!s->fin_vel) TRY(dalloc(s, &s->fin_vel, 3 * N));
    if (!s->adj_f[0])
        for (int k = 0; k < 4; ++k) TRY(dalloc(s, &s->adj_f[k], 3 * N));
    if (!s->fin_X || !s->lamX) {
        TRY(dalloc(s, &s->fin_X, 3 * (size_t)M));
        TRY(dalloc(s, &s->lamX, 3 * (size_t)M));
        TRY(dalloc(s, &s->lamXh, 3 * (size_t)M));
        TRY(dalloc(s, &s->mbar1, 3 * (size_t)M));
        TRY(dalloc(s, &s->mbar2, 3 * (size_t)M));
        TRY(dalloc(s, &s->lamG, 3 * (size_t)M));
        TRY(dalloc(s, &s->Gtmp, 3 * (size_t)M));
        TRY(dalloc(s, &s->Ubuf, 3 * (size_t)M));
        TRY(dalloc(s, &s->dkp, (size_t)M));
    }
    return AFMIB_OK;
}

int traj_forward(afmib_solver* s, int nsteps, int every) {
    if (s->d.channel) return s->fail(AFMIB_ERR_ARG, "the adjoint trajectory needs the periodic domain");
    if (s->d.nz == 1) return s->fail(AFMIB_ERR_ARG, "the adjoint trajectory needs a 3D grid");
    if (s->M <= 0) return s->fail(AFMIB_ERR_STATE, "no markers set");
    if (!s->nbr_symmetric) return s->fail(AFMIB_ERR_ARG, "the adjoint needs symmetric spring neighbour lists");
    if (s->has_vol) return s->fail(AFMIB_ERR_ARG, "the adjoint uses unit marker volumes");
    if (nsteps < 1 || every < 1) return s->fail(AFMIB_ERR_ARG, "nsteps and every must be positive");
    TRY(traj_alloc(s, nsteps, every));
    const size_t mb = 3 * (size_t)s->M * sizeof(double);
    // cold-started projections, so that the reverse pass recomputes every
    // segment exactly from its checkpoint
    const bool warm = s->warm_start;
    s->warm_start = false;
    struct Restore { afmib_solver* s; bool w; ~Restore() { s->warm_start = w; } } restore{s, warm};
    for (int st = 0; st < nsteps; ++st) {
        if (st % every == 0) {
            TRY(copy_vel_out(s, s->ck_vel[st / every]));
            CK(cudaMemcpyAsync(s->ck_X[st / every], s->X, mb, cudaMemcpyDeviceToDevice, s->st));
        }
        TRY(ib_one_step(s));
    }
    TRY(copy_vel_out(s, s->fin_vel));
    CK(cudaMemcpyAsync(s->fin_X, s->X, mb, cudaMemcpyDeviceToDevice, s->st));
    s->traj_steps = nsteps;
    s->traj_every = every;
    return sync(s);
}

// FP64 marker forces G (per component) at positions P: springs, plus bending
// when the configuration has it
void marker_forces(afmib_solver* s, const double* P, double* G) {
    if (s->cfg.k_bend != 0.0)
        launch_springs_bending<double>(s->M, P, s->nstart, s->nidx, s->cfg.k_spring, s->cfg.k_bend, s->Ybend, G, s->st);
    else
        launch_springs<double>(s->M, P, s->nstart, s->nidx, s->cfg.k_spring, G, s->st);
}

// Reverse of one IB step over record j: (L = lam_u^{n+1}, lamX = lam_X^{n+1})
// -> (lam_u^n, lam_X^n), lam_k accumulated in *lam_k.
int adjoint_step(afmib_solver* s, int j, double* lam_k) {
    const Dims& d = s->d;
    const long long N = s->N();
    const int M = s->M;
    const double dt = s->cfg.dt, rho = s->cfg.rho, kk = s->cfg.k_spring;
    const double n3 = (double)d.n * d.n * d.n;
    double* L = s->adj_f[0];
    double* A = s->adj_f[1];
    double* T = s->adj_f[2];
    double* R = s->adj_f[3];
    const double* u0 = s->rec_u0[j];
    const double* uh = s->rec_uh[j];
    const double* X0 = s->rec_X0[j];
    const double* Xh = s->rec_Xh[j];
    auto F = [&](double* b, int c) { return b + c * N; };
    auto cF = [&](const double* b, int c) { return b + c * N; };
    // lam_U2 = dt lam_X1
    launch_aos_to_soa(M, s->lamX, s->mbar2, dt, s->st);
    // ---- CN: u1 = P H^{-1} (H+ u0 + dt (fh/rho - N(uh)))
    CK(cudaMemcpyAsync(T, L, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    TRY(project_fields(s, F(T, 0), F(T, 1), F(T, 2)));
    TRY(helm_inverse(s, R, T));
    for (int c = 0; c < 3; ++c) launch_helm_apply<double>(d, c, s->s_plus(), F(A, c), F(R, c), s->st);
    // lam_uh = N'(uh)^T (-dt R)
    CK(cudaMemsetAsync(T, 0, 3 * N * sizeof(double), s->st));
    launch_axpy<double>(3 * N, T, R, -dt, s->st);
    {
        ProfScope ps(s, P_ADJ_ADVECT, 12.0 * N * 8);
        launch_advect_adjoint(d, F(L, 0), F(L, 1), F(L, 2), cF(uh, 0), cF(uh, 1), cF(uh, 2), F(T, 0), F(T, 1),
                              F(T, 2), 0, s->st);
    }
    CKL();
    // fh = S(Xh) Gh with Gh = k K Xh; lam_fh = (dt/rho) R
    TRY(bin_markers(s, Xh, false));
    marker_forces(s, Xh, s->Gtmp);
    TRY(interp_markers(s, F(R, 0), F(R, 1), F(R, 2), s->Ubuf, false));
    CK(cudaMemsetAsync(s->lamG, 0, 3 * (size_t)M * sizeof(double), s->st));
    launch_axpy<double>(3 * (long long)M, s->lamG, s->Ubuf, n3 * dt / rho, s->st);
    CK(cudaMemsetAsync(s->lamXh, 0, 3 * (size_t)M * sizeof(double), s->st));
    {
        ProfScope ps(s, P_ADJ_MARKER, (double)M * 400, 2);
        launch_marker_grad(d, M, Xh, s->Gtmp, F(R, 0), F(R, 1), F(R, 2), n3 * dt / rho, s->lamXh, s->st);
        launch_springs_adjoint(M, Xh, s->nstart, s->nidx, kk, s->lamG, s->lamXh, s->dkp, s->st);
        if (s->cfg.k_bend != 0.0)
            launch_bending_adjoint(M, s->nstart, s->nidx, s->cfg.k_bend, s->lamG, s->Ybend, s->lamXh, s->st);
    }
    launch_sum<double>(M, s->dkp, s->red, s->scal + 11, s->st);
    CKL();
    TRY(read_scalars(s, 11, 1));
    *lam_k += s->hscal[11];
    // U2 = I(Xh) uh
    TRY(spread_generic(s, s->mbar2, nullptr, 1.0, F(T, 0), F(T, 1), F(T, 2)));
    launch_axpy<double>(3 * N, L, T, 1.0, s->st);
    launch_marker_grad(d, M, Xh, s->mbar2, cF(uh, 0), cF(uh, 1), cF(uh, 2), 1.0, s->lamXh, s->st);
    // Xh = X0 + dt/2 U1: lam_X0 += lam_Xh, lam_U1 = dt/2 lam_Xh
    launch_axpy<double>(3 * (long long)M, s->lamX, s->lamXh, 1.0, s->st);
    launch_aos_to_soa(M, s->lamXh, s->mbar1, dt / 2, s->st);
    // U1 = I(X0) uh
    TRY(bin_markers(s, X0, false));
    TRY(spread_generic(s, s->mbar1, nullptr, 1.0, F(T, 0), F(T, 1), F(T, 2)));
    launch_axpy<double>(3 * N, L, T, 1.0, s->st);
    launch_marker_grad(d, M, X0, s->mbar1, cF(uh, 0), cF(uh, 1), cF(uh, 2), 1.0, s->lamX, s->st);
    // ---- BE: uh = P H^{-1} (u0 + dt/2 (f0/rho - N(u0)))
    CK(cudaMemcpyAsync(T, L, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    TRY(project_fields(s, F(T, 0), F(T, 1), F(T, 2)));
    TRY(helm_inverse(s, R, T));
    launch_axpy<double>(3 * N, A, R, 1.0, s->st);
    CK(cudaMemsetAsync(T, 0, 3 * N * sizeof(double), s->st));
    launch_axpy<double>(3 * N, T, R, -dt / 2, s->st);
    {
        ProfScope ps(s, P_ADJ_ADVECT, 12.0 * N * 8);
        launch_advect_adjoint(d, F(A, 0), F(A, 1), F(A, 2), cF(u0, 0), cF(u0, 1), cF(u0, 2), F(T, 0), F(T, 1),
                              F(T, 2), 1, s->st);
    }
    // f0 = S(X0) G0, lam_f0 = dt/(2 rho) R (bins of X0 are current)
    marker_forces(s, X0, s->Gtmp);
    TRY(interp_markers(s, F(R, 0), F(R, 1), F(R, 2), s->Ubuf, false));
    CK(cudaMemsetAsync(s->lamG, 0, 3 * (size_t)M * sizeof(double), s->st));
    launch_axpy<double>(3 * (long long)M, s->lamG, s->Ubuf, n3 * dt / (2 * rho), s->st);
    {
        ProfScope ps(s, P_ADJ_MARKER, (double)M * 400, 2);
        launch_marker_grad(d, M, X0, s->Gtmp, F(R, 0), F(R, 1), F(R, 2), n3 * dt / (2 * rho), s->lamX, s->st);
        launch_springs_adjoint(M, X0, s->nstart, s->nidx, kk, s->lamG, s->lamX, s->dkp, s->st);
        if (s->cfg.k_bend != 0.0)
            launch_bending_adjoint(M, s->nstart, s->nidx, s->cfg.k_bend, s->lamG, s->Ybend, s->lamX, s->st);
    }
    launch_sum<double>(M, s->dkp, s->red, s->scal + 11, s->st);
    CKL();
    TRY(read_scalars(s, 11, 1));
    *lam_k += s->hscal[11];
    CK(cudaMemcpyAsync(L, A, 3 * N * sizeof(double), cudaMemcpyDeviceToDevice, s->st));
    return AFMIB_OK;
}

int traj_adjoint(afmib_solver* s, const double* lu, const double* lv, const double* lw, const double* lX,
                 double* gX0, double* gk, double* gu0, double* gv0, double* gw0) {
    if (s->traj_steps <= 0) return s->fail(AFMIB_ERR_STATE, "no trajectory: call afmib_trajectory_forward first");
    const long long N = s->N();
    const int M = s->M;
    const size_t mb = 3 * (size_t)M * sizeof(double);
    double* L = s->adj_f[0];
    TRY(copy_in(s, L, lu, N));
    TRY(copy_in(s, L + N, lv, N));
    TRY(copy_in(s, L + 2 * N, lw, N));
    TRY(copy_in(s, s->lamX, lX, 3 * (long long)M));
    // The adjoint is linear in (lam_u, lam_X), but its solves stop on the
    // forward's absolute tolerances, which only mean something for fields of
    // the forward's magnitude: a loss term like h^3 |u|^2 gives cotangents of
    // order h^3 (1e-9 at 512^3), against which a tolerance of 1e-10 is no
    // convergence at all. So the cotangents are scaled to unit RMS on the way
    // in and the gradients scaled back on the way out.
    launch_sumsq<double>(3 * N, L, s->red, s->scal + 16, s->st);
    launch_sumsq<double>(3 * (long long)M, s->lamX, s->red, s->scal + 17, s->st);
    CKL();
    TRY(read_scalars(s, 16, 2));
    const double rms = std::max(std::sqrt(s->hscal[16] / (3.0 * (double)N)),
                                M > 0 ? std::sqrt(s->hscal[17] / (3.0 * (double)M)) : 0.0);
    const char* es = std::getenv("AFMIB_ADJ_SCALE");  // 0: unscaled (for comparison)
    const bool scale_on = !(es && es[0] == '0');
    const double sigma = (scale_on && rms > 0.0 && std::isfinite(rms)) ? 1.0 / rms : 1.0;
    if (sigma != 1.0) {
        launch_scale<double>(3 * N, L, sigma, s->st);
        launch_scale<double>(3 * (long long)M, s->lamX, sigma, s->st);
    }
    double lam_k = 0.0;
    const bool warm = s->warm_start;
    s->warm_start = false;
    struct Restore { afmib_solver* s; bool w; ~Restore() { s->warm_start = w; } } restore{s, warm};
    const int nseg = (s->traj_steps + s->traj_every - 1) / s->traj_every;
    const bool half_saved = s->half;
    for (int sg = nseg - 1; sg >= 0; --sg) {
        const int first = sg * s->traj_every;
        const int cnt = std::min(s->traj_every, s->traj_steps - first);
        TRY(copy_vel_in(s, s->ck_vel[sg]));
        CK(cudaMemcpyAsync(s->X, s->ck_X[sg], mb, cudaMemcpyDeviceToDevice, s->st));
        s->recording = true;
        for (int j = 0; j < cnt; ++j) {
            s->rec_j = j;
            const int rc = ib_one_step(s);
            if (rc != AFMIB_OK) { s->recording = false; return rc; }
        }
        s->recording = false;
        for (int j = cnt - 1; j >= 0; --j) TRY(adjoint_step(s, j, &lam_k));
    }
    // leave the solver at the end state of the trajectory
    TRY(copy_vel_in(s, s->fin_vel));
    CK(cudaMemcpyAsync(s->X, s->fin_X, mb, cudaMemcpyDeviceToDevice, s->st));
    s->half = half_saved;
    if (sigma != 1.0) {
        launch_scale<double>(3 * N, L, 1.0 / sigma, s->st);
        launch_scale<double>(3 * (long long)M, s->lamX, 1.0 / sigma, s->st);
        lam_k /= sigma;
    }
    TRY(copy_out(s, gX0, s->lamX, 3 * (long long)M));
    TRY(copy_out(s, gu0, L, N));
    TRY(copy_out(s, gv0, L + N, N));
    TRY(copy_out(s, gw0, L + 2 * N, N));
    TRY(sync(s));
    if (gk) *gk = lam_k;
    return AFMIB_OK;
}

int setup_tiles(afmib_solver* s) {
    const Dims& d = s->d;
    // 2D grids (nz == 1) use tiles one cell deep
    const bool flat = d.nz == 1;
    auto ok = [&](int ts) {
        return d.nx % ts == 0 && d.ny % ts == 0 && d.nx >= ts + 4 && d.ny >= ts + 4 &&
               (flat || (d.nz % ts == 0 && d.nz >= ts + 4));
    };
    if (ok(8)) s->TS = 8;
    else if (ok(4)) s->TS = 4;
    else return s->fail(AFMIB_ERR_ARG, "immersed boundary needs every extent a multiple of 4 and at least 8 cells");
    s->TZ = flat ? 1 : s->TS;
    s->ntx = d.nx / s->TS;
    s->nty = d.ny / s->TS;
    s->ntz = d.nz / s->TZ;
    s->ntiles = s->ntx * s->nty * s->ntz;
    TRY(dalloc(s, &s->tstart, s->ntiles));
    TRY(dalloc(s, &s->tend, s->ntiles));
    TRY(dalloc(s, &s->tlist, s->ntiles));
    TRY(dalloc(s, &s->tcount, 5));
    TRY(dalloc(s, &s->tovf, s->ntiles));
    TRY(dalloc(s, &s->tslot, s->ntiles));
    TRY(dalloc(s, &s->tocc, s->ntiles));
    return AFMIB_OK;
}

int create(afmib_solver* s, const afmib_config* c, void* stream) {
    s->cfg = *c;
    afmib_config& g = s->cfg;
    mg_kernel_attributes();  // before any capture of the V-cycles
    if (g.n <= 0) g.n = g.nx;
    if (g.nu1 <= 0) g.nu1 = 2;
    if (g.nu2 <= 0) g.nu2 = 2;
    if (g.max_cg_iters <= 0) g.max_cg_iters = 1000;
    if (g.max_mg_cycles <= 0) g.max_mg_cycles = 200;
    if (g.inner_tol <= 0) g.inner_tol = 1e-5;
    if (g.nx < 2 || g.ny < 2 || g.nz < 1 || (g.nz == 1 && g.bc != AFMIB_BC_PERIODIC))
        return s->fail(AFMIB_ERR_ARG, "extents must be at least 2 cells (nz = 1, a 2D grid, only with periodic bc)");
    // the grid-wide sums keep one partial per block of (32 x 8)-cell tiles
    if ((long long)((g.nx + kRBX - 1) / kRBX) * ((g.ny + kRBY - 1) / kRBY) > kMaxRedBlocks)
        return s->fail(AFMIB_ERR_ARG, "an (x, y) plane of more than 8192 tiles of 32 x 8 cells");
    if (g.bc != AFMIB_BC_PERIODIC && g.bc != AFMIB_BC_CHANNEL) return s->fail(AFMIB_ERR_ARG, "bc must be periodic or channel");
    if (g.precision != AFMIB_FP64 && g.precision != AFMIB_MIXED) return s->fail(AFMIB_ERR_ARG, "precision");
    s->mixed = g.precision == AFMIB_MIXED;
    s->spread64 = s->mixed && !(g.ib_fp32 & 1);
    s->interp64 = s->mixed && !(g.ib_fp32 & 2);
    if (const char* e = std::getenv("AFMIB_SMOOTHER")) s->pipe_smoother = std::string(e) == "pipe";
    if (const char* e = std::getenv("AFMIB_PIPE_MIN_NX")) s->pipe_min_nx = std::atoi(e);
    if (const char* e = std::getenv("AFMIB_BFP")) s->bfp_defects = std::string(e) == "1";
    if (const char* e = std::getenv("AFMIB_INNER_CYCLES"))
        s->inner_cycles = std::min(kMaxInnerCycles, std::max(1, std::atoi(e)));
    if (const char* e = std::getenv("AFMIB_INNER_ADAPT")) s->adapt_cycles = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_INNER_OMEGA")) s->inner_omega = std::atof(e);
    if (const char* e = std::getenv("AFMIB_INNER_NU")) {
        int a = 0, b = 0;
        if (std::sscanf(e, "%d,%d", &a, &b) == 2 && a >= 0 && b >= 0 && a + b > 0) {
            s->inner_nu1 = s->inner_nu1c = a;
            s->inner_nu2 = s->inner_nu2c = b;
        }
    }
    if (const char* e = std::getenv("AFMIB_INNER_NU_COARSE")) {
        int a = 0, b = 0;
        if (std::sscanf(e, "%d,%d", &a, &b) == 2 && a >= 0 && b >= 0 && a + b > 0) {
            s->inner_nu1c = a;
            s->inner_nu2c = b;
        }
    }
    if (const char* e = std::getenv("AFMIB_INNER_SOLVER")) {
        s->jacobi_inner = std::string(e) != "cg";
        s->gs_inner = std::string(e) == "gs";
    }
    if (const char* e = std::getenv("AFMIB_WARM_EXTRAP")) s->warm_extrap = std::string(e) == "1";
    if (const char* e = std::getenv("AFMIB_GRAPHS")) s->use_graphs = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_ALTERNATE")) s->alternate = std::string(e) != "0";
    if (g.walls_corrected != 0 && g.walls_corrected != 1) return s->fail(AFMIB_ERR_ARG, "walls_corrected must be 0 or 1");
    if (g.proj_start < AFMIB_START_DEFAULT || g.proj_start > AFMIB_START_WARM)
        return s->fail(AFMIB_ERR_ARG, "proj_start must be AFMIB_START_DEFAULT, _ZERO or _WARM");
    s->warm_start = g.proj_start == AFMIB_START_WARM || (g.proj_start == AFMIB_START_DEFAULT && s->mixed);
    if (!(g.rho > 0) || !(g.dt > 0) || !(g.mu >= 0) || !(g.tol > 0)) return s->fail(AFMIB_ERR_ARG, "mu, rho, dt, tol");
    s->d = Dims{g.nx, g.ny, g.nz, g.n, g.bc == AFMIB_BC_CHANNEL ? 1 : 0};
    if (stream) {
        s->st = (cudaStream_t)stream;
    } else {
        CK(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    const long long N = s->N();
    TRY(dalloc(s, &s->u, N));
    TRY(dalloc(s, &s->v, N));
    TRY(dalloc(s, &s->w, N));
    for (int k = 0; k < 3; ++k) {
        TRY(dalloc(s, &s->uo[k], N));
        TRY(dalloc(s, &s->adv[k], N));
        TRY(dalloc(s, &s->rhs[k], N));
        TRY(dalloc(s, &s->f[k], N));
        TRY(dalloc(s, &s->tmp[k], N));
    }
    TRY(dalloc(s, &s->divb, N));
    if (const char* e = std::getenv("AFMIB_FUSED_RHS")) s->fused_rhs = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_HELM_OVERLAP")) s->helm_overlap = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_HELM_DF")) s->helm_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_LAP_DF")) s->lap_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_SPREAD_DF")) s->spread_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_INTERP_DF")) s->interp_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_SHADOW_ROUND")) s->round_shadow = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_ADVECT64")) s->advect64 = std::string(e) == "1";
    if (const char* e = std::getenv("AFMIB_ADVECT_DF")) s->advect_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_FIRST_DF")) s->first_df = std::string(e) == "1";
    if (const char* e = std::getenv("AFMIB_PROJ_DF")) s->proj_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_INTERP_PAIRS")) s->interp_pairs = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_PREP_DF")) s->prep_df = std::string(e) != "0";
    if (const char* e = std::getenv("AFMIB_CN_START_OLD")) s->cn_start_old = std::string(e) != "0";
    if (s->mixed && s->fused_rhs)
        for (auto& q : s->qo) TRY(dalloc(s, &q, N));
    TRY(dalloc(s, &s->phi_prev[0], N));
    TRY(dalloc(s, &s->phi_prev[1], N));
    if (s->warm_extrap) {
        TRY(dalloc(s, &s->phi_prev2[0], N));
        TRY(dalloc(s, &s->phi_prev2[1], N));
    }
    TRY(dalloc(s, &s->walls, 4 * s->nxz()));
    TRY(dalloc(s, &s->wallgrad, 8 * s->nxz()));
    TRY(dalloc(s, &s->cg_r, N));
    TRY(dalloc(s, &s->cg_p, N));
    TRY(dalloc(s, &s->cg_q, N));
    TRY(dalloc(s, &s->red.partial, (size_t)kMaxRedBlocks * kMaxRedVals));
    TRY(dalloc(s, &s->red.ticket, 1));
    TRY(dalloc(s, &s->scal, 24));
    TRY(dalloc(s, &s->dflag, 4));
    CK(cudaMallocHost((void**)&s->hscal, 24 * sizeof(double)));
    CK(cudaMallocHost((void**)&s->hflag, 4 * sizeof(int)));
    CK(cudaMemsetAsync(s->red.ticket, 0, sizeof(unsigned), s->st));
    CK(cudaMemsetAsync(s->dflag, 0, 4 * sizeof(int), s->st));
    CK(cudaMemsetAsync(s->walls, 0, 4 * s->nxz() * sizeof(double), s->st));
    CK(cudaMemsetAsync(s->wallgrad, 0, 8 * s->nxz() * sizeof(double), s->st));
    CK(cudaMemsetAsync(s->u, 0, N * sizeof(double), s->st));
    CK(cudaMemsetAsync(s->v, 0, N * sizeof(double), s->st));
    CK(cudaMemsetAsync(s->w, 0, N * sizeof(double), s->st));
    for (int k = 0; k < 3; ++k) CK(cudaMemsetAsync(s->f[k], 0, N * sizeof(double), s->st));

    // multigrid hierarchy
    int levels = g.mg_levels;
    if (levels <= 0) {
        levels = 0;
        Dims t = s->d;
        // 2D grids (nz == 1) coarsen x and y only
        const bool flat = t.nz == 1;
        while (is_even(t.nx) && is_even(t.ny) && (flat || is_even(t.nz)) && t.nx >= 2 && t.ny >= 2 &&
               (flat || t.nz >= 2)) {
            t.nx /= 2; t.ny /= 2; if (!flat) t.nz /= 2; t.n /= 2;
            ++levels;
            if (t.nx == 1 || t.ny == 1 || (!flat && t.nz == 1)) break;
        }
    }
    Dims t = s->d;
    for (int l = 0; l <= levels; ++l) {
        if (l > 0) {
            const bool flat = t.nz == 1;
            if (!is_even(t.nx) || !is_even(t.ny) || !(flat || is_even(t.nz)))
                return s->fail(AFMIB_ERR_ARG, "mg_levels exceeds the number of halvings of the grid");
            t.nx /= 2; t.ny /= 2; if (!flat) t.nz /= 2; t.n = t.n / 2 > 0 ? t.n / 2 : 1;
        }
        MGLevel L{t, nullptr, nullptr, nullptr, nullptr};
        const long long n = t.ncell();
        TRY(dalloc(s, &L.x, n));
        TRY(dalloc(s, &L.b, n));
        TRY(dalloc(s, &L.r, n));
        if (s->pipe_smoother && t.nx >= s->pipe_min_nx) L.pc = rbgs_pipe_cfg<double>(t);
        if (L.pc.FY) TRY(dalloc(s, &L.x2, n));
        s->lv.push_back(L);
    }
    // smoothed levels need even extents for the red-black colouring
    for (size_t l = 0; l + 1 < s->lv.size(); ++l) {
        const Dims& q = s->lv[l].d;
        if (!is_even(q.nx)) return s->fail(AFMIB_ERR_ARG, "smoothed multigrid levels need an even x extent");
    }
    const long long nc = s->lv.back().d.ncell();
    TRY(dalloc(s, &s->cw_p, nc));
    TRY(dalloc(s, &s->cw_q, nc));
    if (s->mixed) {
        for (int k = 0; k < 3; ++k) {
            TRY(dalloc(s, &s->adv32[k], N));
            TRY(dalloc(s, &s->f32[k], N));
            CK(cudaMemsetAsync(s->f32[k], 0, N * sizeof(float), s->st));
        }
        TRY(dalloc(s, &s->d32, N));
        TRY(dalloc(s, &s->e32, N));
        s->d32c[0] = s->d32;
        if (s->lap_df) TRY(dalloc(s, &s->plo, N));
        if (s->helm_overlap) {
            TRY(dalloc(s, &s->d32c[1], N));
            TRY(dalloc(s, &s->d32c[2], N));
            if (s->helm_df) {
                for (int k = 0; k < 3; ++k) TRY(dalloc(s, &s->rlo[k], N));
                TRY(dalloc(s, &s->red2.partial, (size_t)kMaxRedBlocks * kMaxRedVals));
                TRY(dalloc(s, &s->red2.ticket, 1));
                CK(cudaMemsetAsync(s->red2.ticket, 0, sizeof(unsigned), s->st));
            }
            CK(cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking));
            int least = 0, greatest = 0;
            CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            CK(cudaStreamCreateWithPriority(&s->hi, cudaStreamNonBlocking, greatest));
            CK(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
            for (int k = 0; k < 3; ++k) {
                CK(cudaEventCreateWithFlags(&s->ev_def[k], cudaEventDisableTiming));
                CK(cudaEventCreateWithFlags(&s->ev_cor[k], cudaEventDisableTiming));
            }
            int dev = 0, sms = 0;
            CK(cudaGetDevice(&dev));
            CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            int per_sm = 3;
            if (const char* e = std::getenv("AFMIB_HELM_WALK_BLOCKS")) per_sm = std::max(1, std::min(8, std::atoi(e)));
            s->walk_blocks = per_sm * sms;
            int per_sm_be = per_sm;
            if (const char* e = std::getenv("AFMIB_HELM_WALK_BLOCKS_BE")) per_sm_be = std::max(1, std::min(8, std::atoi(e)));
            s->walk_blocks_be = per_sm_be * sms;
        }
        TRY(dalloc(s, &s->u32, N));
        TRY(dalloc(s, &s->v32, N));
        TRY(dalloc(s, &s->w32, N));
        CK(cudaMemsetAsync(s->u32, 0, N * sizeof(float), s->st));
        CK(cudaMemsetAsync(s->v32, 0, N * sizeof(float), s->st));
        CK(cudaMemsetAsync(s->w32, 0, N * sizeof(float), s->st));
        if (s->advect_df && !s->advect64) {
            TRY(dalloc(s, &s->u32l, N));
            TRY(dalloc(s, &s->v32l, N));
            TRY(dalloc(s, &s->w32l, N));
            CK(cudaMemsetAsync(s->u32l, 0, N * sizeof(float), s->st));
            CK(cudaMemsetAsync(s->v32l, 0, N * sizeof(float), s->st));
            CK(cudaMemsetAsync(s->w32l, 0, N * sizeof(float), s->st));
        }
        TRY(dalloc(s, &s->cg32_r, N));
        TRY(dalloc(s, &s->cg32_p, N));
        TRY(dalloc(s, &s->cg32_q, N));
        TRY(dalloc(s, &s->cg32_p2, N));
        for (const MGLevel& L : s->lv) {
            MGLevelT<float> F{L.d, nullptr, nullptr, nullptr, nullptr};
            TRY(dalloc(s, &F.x, L.d.ncell()));
            TRY(dalloc(s, &F.b, L.d.ncell()));
            TRY(dalloc(s, &F.r, L.d.ncell()));
            if (s->pipe_smoother && L.d.nx >= s->pipe_min_nx) F.pc = rbgs_pipe_cfg<float>(L.d);
            if (F.pc.FY) TRY(dalloc(s, &F.x2, L.d.ncell()));
            s->lv32.push_back(F);
        }
        TRY(dalloc(s, &s->cx64, nc));
        TRY(dalloc(s, &s->cb64, nc));
        TRY(dalloc(s, &s->cr64, nc));
    }
    // V-cycle tail, when it leaves at least one smoothed level above the
    // coarsest: in one block from the first level of at most 16^3 cells, or
    // (AFMIB_MG_TAIL_CLUSTER=n) on a cluster of n CTAs from the first level of
    // at most 32^3
    {
        bool tail = true;
        if (const char* e = std::getenv("AFMIB_MG_TAIL")) tail = std::string(e) != "0";
        // the cluster form is opt-in: at 256^3 it measured 114 us per V-cycle
        // for the levels 32^3..1 on 16 CTAs against 80 us for 16^3..1 in one
        // block plus the 32^3 level launches, 36.2 against 36.45 IB steps/s
        int cs = 1;
        if (const char* e = std::getenv("AFMIB_MG_TAIL_CLUSTER")) {
            cs = std::min(vcycle_tail_cluster_max(), std::max(1, std::atoi(e)));
            cudaGetLastError();
        }
        const long long cells = cs > 1 ? 32768 : 4096;
        for (size_t l = 0; tail && l + 1 < s->lv.size(); ++l)
            if (s->lv[l].d.ncell() <= cells && s->lv.size() - l <= (size_t)kMaxTailLevels) {
                s->tail_level = (int)l;
                s->tail_cluster = cs;
                break;
            }
    }
    CK(cudaStreamSynchronize(s->st));
    return AFMIB_OK;
}

// FP32 copy of the velocity for the mixed form's FP32 stencils
int refresh_shadow(afmib_solver* s) {
    if (!s->mixed) return AFMIB_OK;
    launch_shadow(s->N(), s->u32, s->u, s->st, s->round_shadow, s->u32l);
    launch_shadow(s->N(), s->v32, s->v, s->st, s->round_shadow, s->v32l);
    launch_shadow(s->N(), s->w32, s->w, s->st, s->round_shadow, s->w32l);
    CKL();
    return AFMIB_OK;
}

int check_smoother_flag(afmib_solver* s) {
    CK(cudaMemcpyAsync(s->hflag + 3, s->dflag + 3, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    TRY(sync(s));
    if (s->hflag[3] != 0) return s->fail(AFMIB_ERR_CUDA, "pipelined smoother: a row copy did not complete in time");
    return AFMIB_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
// device -> host copy on the solver's stream (the caller synchronises)
template <typename T>
int to_host(afmib_solver* s, std::vector<T>& h, const T* d, long long n) {
    h.resize((size_t)n);
    if (n > 0) CK(cudaMemcpyAsync(h.data(), d, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, s->st));
    return AFMIB_OK;
}

extern "C" {

const char* afmib_error_string(int status) {
    switch (status) {
        case AFMIB_OK: return "ok";
        case AFMIB_ERR_ARG: return "invalid argument";
        case AFMIB_ERR_CUDA: return "CUDA error";
        case AFMIB_ERR_NOCONV: return "iteration cap reached";
        case AFMIB_ERR_BOUNDS: return "marker too close to a wall";
        case AFMIB_ERR_NAN: return "non-finite value";
        case AFMIB_ERR_STATE: return "call out of order";
        case AFMIB_ERR_CAPACITY: return "a fixed capacity exceeded";
        default: return "unknown status";
    }
}

const char* afmib_last_error(const afmib_solver* s) { return s ? s->err.c_str() : "null solver"; }

int afmib_create(const afmib_config* cfg, void* stream, afmib_solver** out) {
    if (!cfg || !out) return AFMIB_ERR_ARG;
    afmib_solver* s = new afmib_solver();
    const int rc = create(s, cfg, stream);
    *out = s;  // returned even on failure so that afmib_last_error can be read
    return rc;
}

int afmib_destroy(afmib_solver* s) {
    if (!s) return AFMIB_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    for (void* p : s->allocs)
        if (p) cudaFree(p);
    drop_graphs(s);
    for (auto& p : s->prof_pend) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : s->prof_pool) cudaEventDestroy(e);
    if (s->hscal) cudaFreeHost(s->hscal);
    if (s->hflag) cudaFreeHost(s->hflag);
    for (cudaStream_t q : {s->aux, s->hi})
        if (q) {
            cudaStreamSynchronize(q);
            cudaStreamDestroy(q);
        }
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    for (int k = 0; k < 3; ++k) {
        if (s->ev_def[k]) cudaEventDestroy(s->ev_def[k]);
        if (s->ev_cor[k]) cudaEventDestroy(s->ev_cor[k]);
    }
    if (s->own_stream && s->st) cudaStreamDestroy(s->st);
    delete s;
    return AFMIB_OK;
}

int afmib_get_stats(const afmib_solver* s, afmib_stats* out) {
    if (!s || !out) return AFMIB_ERR_ARG;
    *out = s->stats;
    return AFMIB_OK;
}

int afmib_synchronize(afmib_solver* s) {
    if (!s) return AFMIB_ERR_ARG;
    return sync(s);
}

int afmib_set_velocity(afmib_solver* s, const double* u, const double* v, const double* w) {
    if (!s) return AFMIB_ERR_ARG;
    TRY(copy_in(s, s->u, u, s->N()));
    if (v) TRY(v_in(s, s->v, v));
    else CK(cudaMemsetAsync(s->v, 0, s->N() * sizeof(double), s->st));
    TRY(copy_in(s, s->w, w, s->N()));
    TRY(refresh_shadow(s));
    // The warm-start potentials stay: they are only the projections' first
    // guess (the stopping rule is unchanged), and a caller that feeds the
    // velocity back every step (a host-coupled loop) keeps its warm starts.
    // afmib_reset_warm_start drops them for runs that must not depend on the
    // solver's history.
    s->phi_valid2[0] = s->phi_valid2[1] = false;
    s->qo_valid = false;
    return sync(s);
}

int afmib_reset_warm_start(afmib_solver* s) {
    if (!s) return AFMIB_ERR_ARG;
    s->phi_valid[0] = s->phi_valid[1] = false;
    s->phi_valid2[0] = s->phi_valid2[1] = false;
    s->mg_rho = 0.0;
    return AFMIB_OK;
}

int afmib_get_velocity(afmib_solver* s, double* u, double* v, double* w) {
    if (!s) return AFMIB_ERR_ARG;
    TRY(copy_out(s, u, s->u, s->N()));
    if (v) TRY(v_out(s, v, s->v));
    TRY(copy_out(s, w, s->w, s->N()));
    return sync(s);
}

int afmib_get_pressure(afmib_solver* s, double* p) {
    if (!s || !p) return AFMIB_ERR_ARG;
    launch_helm_apply<double>(s->d, 0, s->s_minus(), s->tmp[0], s->lv[0].x, s->st);
    CKL();
    TRY(copy_out(s, p, s->tmp[0], s->N()));
    return sync(s);
}

int afmib_set_walls(afmib_solver* s, const double* ut, const double* ub, const double* wt, const double* wb) {
    if (!s) return AFMIB_ERR_ARG;
    const long long n = s->nxz();
    TRY(copy_in(s, s->walls, ut, n));
    TRY(copy_in(s, s->walls + n, ub, n));
    TRY(copy_in(s, s->walls + 2 * n, wt, n));
    TRY(copy_in(s, s->walls + 3 * n, wb, n));
    return sync(s);
}

int afmib_get_walls(afmib_solver* s, double* ut, double* ub, double* wt, double* wb) {
    if (!s) return AFMIB_ERR_ARG;
    const long long n = s->nxz();
    TRY(copy_out(s, ut, s->walls, n));
    TRY(copy_out(s, ub, s->walls + n, n));
    TRY(copy_out(s, wt, s->walls + 2 * n, n));
    TRY(copy_out(s, wb, s->walls + 3 * n, n));
    return sync(s);
}

int afmib_project(afmib_solver* s) {
    if (!s) return AFMIB_ERR_ARG;
    TRY(project(s));
    return sync(s);
}

int afmib_ns_step(afmib_solver* s, const double* fx, const double* fy, const double* fz) {
    if (!s) return AFMIB_ERR_ARG;
    TRY(copy_in(s, s->f[0], fx, s->N()));
    if (fy) TRY(v_in(s, s->f[1], fy));
    else CK(cudaMemsetAsync(s->f[1], 0, s->N() * sizeof(double), s->st));
    TRY(copy_in(s, s->f[2], fz, s->N()));
    if (s->mixed)
        for (int c = 0; c < 3; ++c) launch_convert<float, double>(s->N(), s->f32[c], s->f[c], s->st);
    CKL();
    TRY(substep(s));
    return sync(s);
}

int afmib_set_markers(afmib_solver* s, int M, const double* X, const int* nstart, const int* nidx, const double* vol) {
    if (!s || M < 0 || (M > 0 && !X)) return AFMIB_ERR_ARG;
    if (!s->TS) TRY(setup_tiles(s));
    int nnz = 0;
    std::vector<int> hstart;
    if (nstart) {
        hstart.resize(M + 1);
        CK(cudaMemcpy(hstart.data(), nstart, (M + 1) * sizeof(int), cudaMemcpyDefault));
        nnz = hstart[M];
        if (hstart[0] != 0 || nnz < 0) return s->fail(AFMIB_ERR_ARG, "nstart must start at 0");
        for (int i = 0; i < M; ++i)
            if (hstart[i + 1] < hstart[i]) return s->fail(AFMIB_ERR_ARG, "nstart must be non-decreasing");
        if (nnz > 0 && !nidx) return s->fail(AFMIB_ERR_ARG, "nidx missing");
        if (nnz > 0) {
            std::vector<int> hidx(nnz);
            CK(cudaMemcpy(hidx.data(), nidx, nnz * sizeof(int), cudaMemcpyDefault));
            for (int e = 0; e < nnz; ++e)
                if (hidx[e] < 0 || hidx[e] >= M) return s->fail(AFMIB_ERR_ARG, "neighbour index out of range");
            // symmetric lists (j in N(i) <=> i in N(j)) make K symmetric, which the adjoint relies on
            std::vector<long long> pairs(nnz);
            for (int i = 0; i < M; ++i)
                for (int e = hstart[i]; e < hstart[i + 1]; ++e) pairs[e] = (long long)i * M + hidx[e];
            std::sort(pairs.begin(), pairs.end());
            bool sym = true;
            for (int i = 0; i < M && sym; ++i)
                for (int e = hstart[i]; e < hstart[i + 1] && sym; ++e)
                    sym = std::binary_search(pairs.begin(), pairs.end(), (long long)hidx[e] * M + i);
            s->nbr_symmetric = sym;
        } else {
            s->nbr_symmetric = true;
        }
    }
    TRY(marker_alloc(s, M, nnz));
    s->M = M;
    TRY(copy_in(s, s->X, X, 3 * (long long)M));
    if (nstart) {
        CK(cudaMemcpyAsync(s->nstart, hstart.data(), (M + 1) * sizeof(int), cudaMemcpyHostToDevice, s->st));
        if (nnz > 0) CK(cudaMemcpyAsync(s->nidx, nidx, nnz * sizeof(int), cudaMemcpyDefault, s->st));
    } else {
        CK(cudaMemsetAsync(s->nstart, 0, (M + 1) * sizeof(int), s->st));
    }
    s->has_vol = vol != nullptr;
    if (vol) TRY(copy_in(s, s->mvol, vol, M));
    return sync(s);
}

int afmib_set_marker_positions(afmib_solver* s, const double* X) {
    if (!s || !X) return AFMIB_ERR_ARG;
    if (s->M <= 0) return s->fail(AFMIB_ERR_STATE, "no markers set");
    TRY(copy_in(s, s->X, X, 3 * (long long)s->M));
    return AFMIB_OK;
}

int afmib_get_markers(afmib_solver* s, double* X) {
    if (!s || !X) return AFMIB_ERR_ARG;
    TRY(copy_out(s, X, s->X, 3 * (long long)s->M));
    return sync(s);
}

// ---------------------------------------------------------------------------
// Snapshots (snapshot_io.h): everything a run needs to continue bit for bit.
// ---------------------------------------------------------------------------
int afmib_save(afmib_solver* s, const char* path) {
    if (!s || !path) return AFMIB_ERR_ARG;
    const long long N = s->N(), nxz = s->nxz(), M = s->M;
    std::vector<double> u, v, w, phi, pp0, pp1, walls, wallgrad, X, vol, uo[3], qo[3];
    std::vector<int> nstart, nidx;
    TRY(to_host(s, u, s->u, N));
    // mid-step (a Crank-Nicolson sub-step next): its right-hand side needs the
    // velocity at the start of the step and, in the mixed form, Q of it
    for (int c = 0; c < 3 && s->half; ++c) {
        TRY(to_host(s, uo[c], s->uo[c], N));
        if (s->qo_valid) TRY(to_host(s, qo[c], s->qo[c], N));
    }
    TRY(to_host(s, v, s->v, N));
    TRY(to_host(s, w, s->w, N));
    TRY(to_host(s, phi, s->lv[0].x, N));
    if (s->phi_valid[0]) TRY(to_host(s, pp0, s->phi_prev[0], N));
    if (s->phi_valid[1]) TRY(to_host(s, pp1, s->phi_prev[1], N));
    TRY(to_host(s, walls, s->walls, 4 * nxz));
    // the wall rows of the last projection's gradient, which the next
    // sub-step's wall update uses (channel)
    TRY(to_host(s, wallgrad, s->wallgrad, 8 * nxz));
    if (M > 0) {
        TRY(to_host(s, X, s->X, 3 * M));
        TRY(to_host(s, nstart, s->nstart, M + 1));
        if (s->has_vol) TRY(to_host(s, vol, s->mvol, M));
    }
    TRY(sync(s));
    if (M > 0 && nstart[M] > 0) {
        TRY(to_host(s, nidx, s->nidx, nstart[M]));
        TRY(sync(s));
    }
    snap::Writer wr;
    wr.h.nx = s->d.nx;
    wr.h.ny = s->d.ny;
    wr.h.nz = s->d.nz;
    wr.h.n = s->d.n;
    wr.h.bc = s->cfg.bc;
    wr.h.precision = s->cfg.precision;
    wr.h.half = s->half ? 1 : 0;
    wr.h.substeps = s->stats.substeps;
    wr.h.mg_rho = s->mg_rho;
    wr.add("u", snap::kF64, u.data(), u.size());
    wr.add("v", snap::kF64, v.data(), v.size());
    wr.add("w", snap::kF64, w.data(), w.size());
    wr.add("phi", snap::kF64, phi.data(), phi.size());
    if (!pp0.empty()) wr.add("phi_prev0", snap::kF64, pp0.data(), pp0.size());
    if (!pp1.empty()) wr.add("phi_prev1", snap::kF64, pp1.data(), pp1.size());
    wr.add("walls", snap::kF64, walls.data(), walls.size());
    wr.add("wallgrad", snap::kF64, wallgrad.data(), wallgrad.size());
    const char* uo_name[3] = {"uo0", "uo1", "uo2"};
    const char* qo_name[3] = {"qo0", "qo1", "qo2"};
    for (int c = 0; c < 3; ++c) {
        if (!uo[c].empty()) wr.add(uo_name[c], snap::kF64, uo[c].data(), uo[c].size());
        if (!qo[c].empty()) wr.add(qo_name[c], snap::kF64, qo[c].data(), qo[c].size());
    }
    if (M > 0) {
        wr.add("X", snap::kF64, X.data(), X.size());
        wr.add("nstart", snap::kI32, nstart.data(), nstart.size());
        wr.add("nidx", snap::kI32, nidx.data(), nidx.size());
        if (s->has_vol) wr.add("vol", snap::kF64, vol.data(), vol.size());
    }
    if (!wr.write(path)) return s->fail(AFMIB_ERR_ARG, "cannot write the snapshot file");
    return AFMIB_OK;
}

int afmib_load(afmib_solver* s, const char* path) {
    if (!s || !path) return AFMIB_ERR_ARG;
    snap::Header h{};
    std::map<std::string, snap::Section> sec;
    const std::string err = snap::read(path, &h, &sec);
    if (!err.empty()) return s->fail(AFMIB_ERR_ARG, err);
    if (h.nx != s->d.nx || h.ny != s->d.ny || h.nz != s->d.nz || h.n != s->d.n || h.bc != s->cfg.bc)
        return s->fail(AFMIB_ERR_ARG, "the snapshot's grid or boundary conditions differ from the solver's");
    const long long N = s->N(), nxz = s->nxz();
    auto f64 = [&](const char* name, long long count) -> const double* {
        auto it = sec.find(name);
        if (it == sec.end() || it->second.dtype != snap::kF64 || (long long)it->second.count() != count) return nullptr;
        return it->second.f64();
    };
    const double *u = f64("u", N), *v = f64("v", N), *w = f64("w", N), *phi = f64("phi", N),
                 *walls = f64("walls", 4 * nxz), *wallgrad = f64("wallgrad", 8 * nxz);
    if (!u || !v || !w || !phi || !walls || !wallgrad)
        return s->fail(AFMIB_ERR_ARG, "snapshot sections missing or of the wrong size");
    CK(cudaMemcpyAsync(s->u, u, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->v, v, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->w, w, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->lv[0].x, phi, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->walls, walls, 4 * nxz * sizeof(double), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->wallgrad, wallgrad, 8 * nxz * sizeof(double), cudaMemcpyHostToDevice, s->st));
    TRY(refresh_shadow(s));
    for (int k = 0; k < 2; ++k) {
        const double* pp = f64(k == 0 ? "phi_prev0" : "phi_prev1", N);
        s->phi_valid[k] = pp != nullptr;
        if (pp) CK(cudaMemcpyAsync(s->phi_prev[k], pp, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
    }
    s->phi_valid2[0] = s->phi_valid2[1] = false;
    s->qo_valid = false;
    if (h.half) {
        const char* uo_name[3] = {"uo0", "uo1", "uo2"};
        const char* qo_name[3] = {"qo0", "qo1", "qo2"};
        bool q_all = s->qo[0] != nullptr;
        for (int c = 0; c < 3; ++c) {
            const double* uo = f64(uo_name[c], N);
            if (!uo) return s->fail(AFMIB_ERR_ARG, "a mid-step snapshot without the step's start velocity");
            CK(cudaMemcpyAsync(s->uo[c], uo, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
            const double* q = f64(qo_name[c], N);
            if (q && s->qo[c]) CK(cudaMemcpyAsync(s->qo[c], q, N * sizeof(double), cudaMemcpyHostToDevice, s->st));
            q_all = q_all && q;
        }
        s->qo_valid = q_all;
    }
    s->half = h.half != 0;
    s->stats.half = h.half;
    s->stats.substeps = h.substeps;
    s->mg_rho = h.mg_rho;
    TRY(sync(s));
    auto xs = sec.find("X");
    if (xs != sec.end()) {
        const long long M = (long long)xs->second.count() / 3;
        auto ns = sec.find("nstart");
        auto ni = sec.find("nidx");
        if (xs->second.dtype != snap::kF64 || ns == sec.end() || ns->second.dtype != snap::kI32 ||
            (long long)ns->second.count() != M + 1 || ni == sec.end() || ni->second.dtype != snap::kI32)
            return s->fail(AFMIB_ERR_ARG, "snapshot marker sections inconsistent");
        const double* vol = f64("vol", M);
        TRY(afmib_set_markers(s, (int)M, xs->second.f64(), ns->second.i32(), ni->second.i32(), vol));
    }
    return AFMIB_OK;
}

int afmib_ib_step(afmib_solver* s, int nsteps) {
    if (!s) return AFMIB_ERR_ARG;
    if (s->M <= 0) return s->fail(AFMIB_ERR_STATE, "no markers set");
    for (int k = 0; k < nsteps; ++k) TRY(ib_one_step(s));
    return AFMIB_OK;
}

// ---- single operators ------------------------------------------------------

int afmib_div(afmib_solver* s, double* dout, const double* u, const double* v, const double* w, const double* top,
              const double* bottom) {
    if (!s || !dout || !u || !v || !w) return AFMIB_ERR_ARG;
    const long long N = s->N(), nxz = s->nxz();
    TRY(copy_in(s, s->tmp[0], u, N));
    TRY(v_in(s, s->tmp[1], v));
    TRY(copy_in(s, s->tmp[2], w, N));
    TRY(copy_in(s, s->adv[0], top, nxz));
    TRY(copy_in(s, s->adv[1], bottom, nxz));
    launch_div<double>(s->d, s->divb, s->tmp[0], s->tmp[1], s->tmp[2], s->adv[0], s->adv[1], s->st);
    CKL();
    TRY(copy_out(s, dout, s->divb, N));
    return sync(s);
}

int afmib_grad(afmib_solver* s, double* px, double* py, double* pz, const double* p) {
    if (!s || !px || !py || !pz || !p) return AFMIB_ERR_ARG;
    const long long N = s->N();
    TRY(copy_in(s, s->divb, p, N));
    CK(cudaMemsetAsync(s->tmp[1], 0, N * sizeof(double), s->st));
    launch_grad<double>(s->d, s->tmp[0], s->tmp[1], s->tmp[2], s->divb, s->st);
    CKL();
    TRY(copy_out(s, px, s->tmp[0], N));
    TRY(v_out(s, py, s->tmp[1]));
    TRY(copy_out(s, pz, s->tmp[2], N));
    return sync(s);
}

int afmib_advection(afmib_solver* s, double* ua, double* va, double* wa, const double* u, const double* v,
                    const double* w) {
    if (!s || !ua || !va || !wa || !u || !v || !w) return AFMIB_ERR_ARG;
    const long long N = s->N();
    TRY(copy_in(s, s->tmp[0], u, N));
    TRY(v_in(s, s->tmp[1], v));
    TRY(copy_in(s, s->tmp[2], w, N));
    launch_advect<double, double>(s->d, s->rhs[0], s->rhs[1], s->rhs[2], s->tmp[0], s->tmp[1], s->tmp[2], s->st);
    CKL();
    TRY(copy_out(s, ua, s->rhs[0], N));
    TRY(v_out(s, va, s->rhs[1]));
    TRY(copy_out(s, wa, s->rhs[2], N));
    return sync(s);
}

int afmib_mg_solve(afmib_solver* s, double* rhs, int* cycles) {
    if (!s || !rhs) return AFMIB_ERR_ARG;
    TRY(copy_in(s, s->lv[0].b, rhs, s->N()));
    const int rc = s->mixed ? mg_solve_mixed(s, cycles) : mg_solve(s, cycles);
    TRY(copy_out(s, rhs, s->lv[0].x, s->N()));
    TRY(sync(s));
    return rc;
}

int afmib_lap_apply(afmib_solver* s, double* y, const double* x) {
    if (!s || !y || !x) return AFMIB_ERR_ARG;
    TRY(copy_in(s, s->tmp[0], x, s->N()));
    launch_lap_apply<double>(s->d, s->tmp[1], s->tmp[0], s->st);
    CKL();
    TRY(copy_out(s, y, s->tmp[1], s->N()));
    return sync(s);
}

int afmib_helm_apply(afmib_solver* s, int comp, double scale, double* y, const double* x) {
    if (!s || !y || !x || comp < 0 || comp > 2) return AFMIB_ERR_ARG;
    if (comp == 1) TRY(v_in(s, s->tmp[0], x));
    else TRY(copy_in(s, s->tmp[0], x, s->N()));
    launch_helm_apply<double>(s->d, comp, scale, s->tmp[1], s->tmp[0], s->st);
    CKL();
    if (comp == 1) TRY(v_out(s, y, s->tmp[1]));
    else TRY(copy_out(s, y, s->tmp[1], s->N()));
    return sync(s);
}

int afmib_helmholtz_cg(afmib_solver* s, int comp, double scale, double* x, const double* b, int* iters) {
    if (!s || !x || !b || comp < 0 || comp > 2) return AFMIB_ERR_ARG;
    if (comp == 1) {
        TRY(v_in(s, s->tmp[0], x));
        TRY(v_in(s, s->tmp[1], b));
    } else {
        TRY(copy_in(s, s->tmp[0], x, s->N()));
        TRY(copy_in(s, s->tmp[1], b, s->N()));
    }
    const int rc = cg_solve(s, comp, scale, s->tmp[0], s->tmp[1], iters);
    if (comp == 1) TRY(v_out(s, x, s->tmp[0]));
    else TRY(copy_out(s, x, s->tmp[0], s->N()));
    TRY(sync(s));
    return rc;
}

int afmib_restrict(afmib_solver* s, double* coarse, const double* fine) {
    if (!s || !coarse || !fine) return AFMIB_ERR_ARG;
    const Dims& d = s->d;
    if (!is_even(d.nx) || !is_even(d.ny) || !(d.nz == 1 || is_even(d.nz))) return s->fail(AFMIB_ERR_ARG, "odd extent");
    const long long nc = s->N() / (d.nz == 1 ? 4 : 8);
    TRY(copy_in(s, s->tmp[0], fine, s->N()));
    launch_restrict<double>(d, s->tmp[1], s->tmp[0], s->st);
    CKL();
    TRY(copy_out(s, coarse, s->tmp[1], nc));
    return sync(s);
}

int afmib_prolong(afmib_solver* s, double* fine, const double* coarse) {
    if (!s || !coarse || !fine) return AFMIB_ERR_ARG;
    const Dims& d = s->d;
    if (!is_even(d.nx) || !is_even(d.ny) || !(d.nz == 1 || is_even(d.nz))) return s->fail(AFMIB_ERR_ARG, "odd extent");
    TRY(copy_in(s, s->tmp[0], coarse, s->N() / (d.nz == 1 ? 4 : 8)));
    launch_prolong_assign<double>(d, s->tmp[1], s->tmp[0], s->st);
    CKL();
    TRY(copy_out(s, fine, s->tmp[1], s->N()));
    return sync(s);
}

int afmib_spread(afmib_solver* s, int M, const double* X, const double* F, const double* vol, double* fx, double* fy,
                 double* fz) {
    if (!s || M <= 0 || !X || !F || !fx || !fy || !fz) return AFMIB_ERR_ARG;
    if (!s->TS) TRY(setup_tiles(s));
    const int keepM = s->M;
    TRY(marker_alloc(s, M, 0));
    s->M = M;
    TRY(copy_in(s, s->Xh, X, 3 * (long long)M));
    TRY(copy_in(s, s->G, F, 3 * (long long)M));
    if (vol) TRY(copy_in(s, s->U1, vol, M));
    CK(cudaMemsetAsync(s->dflag, 0, sizeof(int), s->st));
    TRY(bin_markers(s, s->Xh));
    TRY(spread_forces(s, vol ? s->U1 : nullptr, s->tmp[0], s->tmp[1], s->tmp[2]));
    int rc = check_marker_flag(s);
    s->M = keepM;
    TRY(copy_out(s, fx, s->tmp[0], s->N()));
    TRY(v_out(s, fy, s->tmp[1]));
    TRY(copy_out(s, fz, s->tmp[2], s->N()));
    TRY(sync(s));
    return rc;
}

int afmib_interp(afmib_solver* s, int M, const double* X, const double* u, const double* v, const double* w,
                 double* U) {
    if (!s || M <= 0 || !X || !u || !v || !w || !U) return AFMIB_ERR_ARG;
    if (!s->TS) TRY(setup_tiles(s));
    const int keepM = s->M;
    TRY(marker_alloc(s, M, 0));
    s->M = M;
    TRY(copy_in(s, s->Xh, X, 3 * (long long)M));
    TRY(copy_in(s, s->tmp[0], u, s->N()));
    TRY(v_in(s, s->tmp[1], v));
    TRY(copy_in(s, s->tmp[2], w, s->N()));
    CK(cudaMemsetAsync(s->dflag, 0, sizeof(int), s->st));
    TRY(bin_markers(s, s->Xh));
    TRY(interp_markers(s, s->tmp[0], s->tmp[1], s->tmp[2], s->U2));
    CKL();
    int rc = check_marker_flag(s);
    s->M = keepM;
    TRY(copy_out(s, U, s->U2, 3 * (long long)M));
    TRY(sync(s));
    return rc;
}

int afmib_set_tolerance(afmib_solver* s, double tol) {
    if (!s || !(tol > 0)) return AFMIB_ERR_ARG;
    if (tol != s->cfg.tol) drop_graphs(s);  // the coarsest solve's tolerance is baked into the graphs
    s->cfg.tol = tol;
    return AFMIB_OK;
}

int afmib_smooth(afmib_solver* s, double* x, const double* b) {
    if (!s || !x || !b) return AFMIB_ERR_ARG;
    MGLevel& L = s->lv[0];
    TRY(copy_in(s, L.x, x, s->N()));
    TRY(copy_in(s, L.b, b, s->N()));
    double* out = L.x;
    if (L.x2 && s->pipe_smoother && L.pc.FY) {
        launch_rbgs_pipe<double>(L.d, L.pc, L.x, L.x2, L.b, s->dflag + 3, s->st);
        out = L.x2;
    } else {
        launch_rbgs<double>(L.d, 0, L.x, L.b, s->st);
        launch_rbgs<double>(L.d, 1, L.x, L.b, s->st);
    }
    CKL();
    TRY(copy_out(s, x, out, s->N()));
    TRY(sync(s));
    return check_smoother_flag(s);
}

int afmib_set_spring(afmib_solver* s, double k) {
    if (!s) return AFMIB_ERR_ARG;
    s->cfg.k_spring = k;
    return AFMIB_OK;
}

int afmib_set_bending(afmib_solver* s, double kb) {
    if (!s) return AFMIB_ERR_ARG;
    s->cfg.k_bend = kb;
    return AFMIB_OK;
}

int afmib_trajectory_forward(afmib_solver* s, int nsteps, int ckpt_every) {
    if (!s) return AFMIB_ERR_ARG;
    return traj_forward(s, nsteps, ckpt_every);
}

int afmib_trajectory_adjoint(afmib_solver* s, const double* lam_u, const double* lam_v, const double* lam_w,
                             const double* lam_X, double* grad_X0, double* grad_k, double* grad_u0, double* grad_v0,
                             double* grad_w0) {
    if (!s) return AFMIB_ERR_ARG;
    return traj_adjoint(s, lam_u, lam_v, lam_w, lam_X, grad_X0, grad_k, grad_u0, grad_v0, grad_w0);
}

// ---- per-kernel profiling ----------------------------------------------------

int afmib_profile_enable(afmib_solver* s, int on) {
    if (!s) return AFMIB_ERR_ARG;
    TRY(sync(s));
    if (s->prof_tab.empty())
        for (int i = 0; i < P_COUNT; ++i) s->prof_tab.push_back({kProfNames[i], 0, 0.0, 0.0});
    s->prof = on != 0;
    return AFMIB_OK;
}

int afmib_profile_reset(afmib_solver* s) {
    if (!s) return AFMIB_ERR_ARG;
    TRY(sync(s));
    for (auto& e : s->prof_tab) { e.launches = 0; e.ms = 0.0; e.bytes = 0.0; }
    return AFMIB_OK;
}

int afmib_profile_count(const afmib_solver* s) { return s ? (int)s->prof_tab.size() : 0; }

int afmib_profile_get(afmib_solver* s, int i, const char** name, long long* launches, double* ms, double* bytes) {
    if (!s || i < 0 || i >= (int)s->prof_tab.size()) return AFMIB_ERR_ARG;
    TRY(sync(s));
    const auto& e = s->prof_tab[i];
    if (name) *name = e.name;
    if (launches) *launches = e.launches;
    if (ms) *ms = e.ms;
    if (bytes) *bytes = e.bytes;
    return AFMIB_OK;
}

}  // extern "C"
