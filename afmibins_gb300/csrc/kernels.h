// Host-side launch wrappers of the afmib sm_103a kernels. Each wrapper
// enqueues on the given stream and returns immediately; T is double (the FP64
// drop-in) or float (the inner passes of the mixed-precision form).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace afmib {

// ----- MAC stencils (kernels_field.cu) -------------------------------------
// Conservative centred advection N(u) of src/ns/solver.h:142-236.
// TI: storage type of the velocity, T: arithmetic and output type.
// The mixed form's advection from the velocity's float pairs (hi, lo), each
// flux difference formed without cancellation (k_advect_df).
void launch_advect_df(const Dims& d, float* ua, float* va, float* wa, const float* uh, const float* ul,
                      const float* vh, const float* vl, const float* wh, const float* wl, cudaStream_t s);
template <typename TI, typename T>
void launch_advect(const Dims& d, T* ua, T* va, T* wa, const TI* u, const TI* v, const TI* w, cudaStream_t s);
// Divergence n*(du + dv + dw), src/alg/div.h:29-60. top/bottom (channel only,
// nx*nz each) may be null for zero walls.
template <typename T>
void launch_div(const Dims& d, T* out, const T* u, const T* v, const T* w, const T* top, const T* bottom,
                cudaStream_t s);
// Mixed form: the divergence in double-float (FP64 in and out, no FP64
// arithmetic but one addition per cell), out_sum[0] = the sum of out.
void launch_div_df(const Dims& d, double* out, const double* u, const double* v, const double* w, const double* top,
                   const double* bottom, RedScratch sc, double* out_sum, cudaStream_t s);
// Gradient onto faces, src/alg/grad.h:29-44 (v plane 0 untouched in channel mode).
template <typename T>
void launch_grad(const Dims& d, T* px, T* py, T* pz, const T* p, cudaStream_t s);
// Projection update u -= grad(phi), src/ns/projection.h:60-73. In channel
// mode the wall-adjacent gradient rows needed by the next wall update are
// saved into wallgrad[8][nx*nz] (may be null): x-gradient at y = 0, 1,
// ny-1, ny-2, z-gradient at y = 0, ny-1, 1, ny-2.
// u32/v32/w32 (optional): FP32 shadow of the updated velocity, rounded to
// nearest (round_shadow) or truncated, by integer operations; with
// u32l/v32l/w32l also the rest of each value's pair (df_split_round).
template <typename T>
void launch_grad_sub(const Dims& d, T* u, T* v, T* w, const T* phi, T* wallgrad, cudaStream_t s, float* u32 = nullptr,
                     float* v32 = nullptr, float* w32 = nullptr, int round_shadow = 1, float* u32l = nullptr,
                     float* v32l = nullptr, float* w32l = nullptr);
// Wall-velocity correction of src/ns/projection.h:75-122 (channel only).
// walls = [ut | ub | wt | wb], nx*nz each.
void launch_wall_update(const Dims& d, double* walls, const double* wallgrad, cudaStream_t s, int corrected = 0);

// Helmholtz right-hand side for one component.
//   be=1: r = u_old - bdy(s_minus) + dt/2 * (f/rho - adv)
//   be=0: r = (I + s_plus*Delta) u_old + bdy(s_plus) - bdy(s_minus) + dt*(f/rho - adv)
// src/ns/solver.h:105-135 with src/ns/helmholtz.h:177-196. walls: [top|bottom]
// rows of this component (null in periodic mode or for v).
// TF: force storage type, TA: advection storage type
template <typename T, typename TF, typename TA>
void launch_helm_rhs(const Dims& d, int comp, int be, T* r, const T* uold, const TF* f, const TA* adv,
                     const double* top, const double* bottom, double s_plus, double s_minus, double dt,
                     double inv_rho, cudaStream_t s);
// Mixed form, backward-Euler sub-step: b (as launch_helm_rhs), the first FP64
// defect r = b - H uold as FP32 with out[0] = r.r (H = I + s_minus Delta), and
// q = Q(uold), the off-diagonal term of the Helmholtz rows, in one pass.
// walk_blocks > 0: the persistent form on that many blocks (tile_walk);
// uo_out: also a copy of uold there; r_lo (the double-float residual): b is
// not written and r is formed as src - bm - off Q.
template <typename TF, typename TA>
void launch_helm_rhs_be_defect(const Dims& d, int comp, double* b, float* r, double* q, const double* uold,
                               const TF* f, const TA* adv, const double* top, const double* bottom, double s_minus,
                               double dt, double inv_rho, RedScratch sc, double* out, cudaStream_t s,
                               int walk_blocks = 0, float* r_lo = nullptr, double* uo_out = nullptr);
// Mixed form, Crank-Nicolson sub-step: b from q = Q(uold) kept by the
// backward-Euler sub-step (pointwise).
template <typename TF, typename TA>
void launch_helm_rhs_cn_q(const Dims& d, int comp, double* r, const double* uold, const double* q, const TF* f,
                          const TA* adv, const double* top, const double* bottom, double s_plus, double s_minus,
                          double dt, double inv_rho, cudaStream_t s);
// Mixed form, Crank-Nicolson sub-step with the double-float residual: x =
// uold and the first residual r = b - H uold from the kept Q (pointwise), as
// its double-float pair (rh, rl), out[0] = rh.rh.
template <typename TF, typename TA>
void launch_helm_cn_first(const Dims& d, int comp, double* x, float* rh, float* rl, const double* uold, const double* q,
                          const TF* f, const TA* adv, const double* top, const double* bottom, double s_plus,
                          double s_minus, double dt, double inv_rho, RedScratch sc, double* out, cudaStream_t s);
// The BE and CN first residuals of the mixed form in double-float on the FP32
// pipe (FP64 forces; the pair form of the residual): the same quantities as
// launch_helm_rhs_be_defect (r_lo given) and launch_helm_cn_first.
template <typename TA>
void launch_helm_rhs_be_defect_df(const Dims& d, int comp, float* r, float* r_lo, double* q, double* uo_out,
                                  const double* uold, const double* f, const TA* adv, const double* top,
                                  const double* bottom, double s_minus, double dt, double inv_rho, RedScratch sc,
                                  double* out, cudaStream_t s, int walk_blocks);
template <typename TA>
void launch_helm_cn_first_df(const Dims& d, int comp, double* x, float* rh, float* rl, const double* uold,
                             const double* q, const double* f, const TA* adv, const double* top, const double* bottom,
                             double s_plus, double s_minus, double dt, double inv_rho, RedScratch sc, double* out,
                             cudaStream_t s);
// Mixed form: r = b - (I + s Delta) x in FP64, stored as TD, out[0] = ||r||^2;
// walk_blocks > 0: the persistent form on that many blocks (tile_walk).
template <typename TD>
void launch_helm_defect(const Dims& d, int comp, double scale, const double* x, const double* b, TD* r, RedScratch sc,
                        double* out, cudaStream_t s, int walk_blocks = 0, float* r_lo = nullptr);
// r_lo (both defects): also the rest of the FP64 residual, float(r - r_float),
// the second word of the double-float pair that launch_helm_update_df updates
// Mixed form: x += e, (rh, rl) -= H e in double-float, out[0] = rh.rh
void launch_helm_update_df(const Dims& d, int comp, double scale, double* x, const float* e, float* rh, float* rl,
                           RedScratch sc, double* out, cudaStream_t s);
// x = 0, r = p = b, cgs[0] = b.b
template <typename T>
void launch_cg_init_zero(long long n, const T* b, T* x, T* r, T* p, RedScratch sc, double* cgs, cudaStream_t s);
// x (FP64) += e
template <typename TE>
void launch_add_correction(long long n, double* x, const TE* e, cudaStream_t s);
// y = (I + s*Delta) x for component comp (src/ns/helmholtz.h:61-175,218-319).
template <typename T>
void launch_helm_apply(const Dims& d, int comp, double scale, T* y, const T* x, cudaStream_t s);

// ----- CG pieces (kernels_field.cu) ------------------------------------------
// Device scalars cgs[] = {n0, pq, n1, beta, alpha} (src/alg/cg.h:36-53).
// init:      r = b - A x, p = r, n0 = r.r
template <typename T>
void launch_cg_init(const Dims& d, int comp, double scale, const T* x, const T* b, T* r, T* p, RedScratch sc,
                    double* cgs, cudaStream_t s);
// apply:     q = A p, pq = p.q, alpha = n0 / pq
template <typename T>
void launch_cg_apply(const Dims& d, int comp, double scale, const T* p, T* q, RedScratch sc, double* cgs,
                     cudaStream_t s);
// update:    x += alpha p, r -= alpha q, n1 = r.r, beta = n1 / n0, n0 = n1
template <typename T>
void launch_cg_update(long long n, T* x, T* r, const T* p, const T* q, RedScratch sc, double* cgs, cudaStream_t s);
// one Jacobi sweep x' = x + (b - H x) / diag(H) (x == nullptr: from zero)
template <typename T>
void launch_helm_jacobi(const Dims& d, int comp, double scale, const T* x, T* xo, const T* b, cudaStream_t s,
                        int rev = 0);
// One colour of a red-black Gauss-Seidel sweep of (I + scale*Delta) x = b in
// place (init: from x = 0). Power-of-two extents, nz a multiple of 8;
// returns false (nothing launched) otherwise.
template <typename T>
bool launch_helm_rbgs(const Dims& d, int comp, double scale, int color, int init, T* x, const T* b, cudaStream_t s,
                      int rev = 0);
// p' = beta p + r formed on the fly (out of place into pn), q = H p', p'.q and alpha
template <typename T>
void launch_cg_dir_apply(const Dims& d, int comp, double scale, const T* p, const T* r, T* pn, T* q, RedScratch sc,
                         double* cgs, cudaStream_t s);
// direction: p = beta p + r
template <typename T>
void launch_cg_direction(long long n, T* p, const T* r, const double* cgs, cudaStream_t s);

// ----- reductions and vector ops (kernels_field.cu) ---------------------------
template <typename T>
void launch_sum(long long n, const T* x, RedScratch sc, double* out, cudaStream_t s);          // sum x
template <typename T>
void launch_sumsq(long long n, const T* x, RedScratch sc, double* out, cudaStream_t s);        // sum x^2
template <typename T>
void launch_sub_scalar_scaled(long long n, T* x, const double* sum, double scale, cudaStream_t s);  // x -= sum*scale
template <typename T>
void launch_fill(long long n, T* x, T value, cudaStream_t s);
template <typename T>
void launch_axpy(long long n, T* y, const T* x, T a, cudaStream_t s);  // y += a x
template <typename T>
void launch_scale(long long n, T* x, T a, cudaStream_t s);  // x *= a
template <typename T>
void launch_lincomb(long long n, T* y, T a, const T* x, T b, const T* z, cudaStream_t s);  // y = a x + b z
// FP32 shadow of an FP64 field, as the projection writes it (rounded to
// nearest by df_round, or truncated by df_hi)
void launch_shadow(long long n, float* out, const double* in, cudaStream_t s, int round_shadow = 1,
                   float* lo = nullptr);
template <typename TO, typename TI>
void launch_convert(long long n, TO* out, const TI* in, cudaStream_t s);

// ----- multigrid (kernels_mg.cu) ---------------------------------------------
// Laplacian n^2*Delta of src/mg/laplacian.h:46-153 (Neumann walls in channel mode).
template <typename T>
void launch_lap_apply(const Dims& d, T* y, const T* x, cudaStream_t s);
// r = b - L x, optionally out[0] = r.r
template <typename T>
void launch_residual(const Dims& d, T* r, const T* x, const T* b, RedScratch* sc, double* out, cudaStream_t s,
                     int rev = 0);
// Mixed form: r = b - L x evaluated in FP64 (x, b FP64), stored as TD; out[0] = r.r
template <typename TD>
void launch_lap_defect(const Dims& d, TD* r, const double* x, const double* b, RedScratch sc, double* out, cudaStream_t s,
                       float* r_lo = nullptr);
// Mixed form: the first defect of a pressure solve in double-float,
// (rh, rl) = (b - sum * scale) - L x (sum null: no mean), out[0] = rh.rh
void launch_lap_defect_df(const Dims& d, float* rh, float* rl, const double* x, const double* b, const double* sum,
                          double scale, RedScratch sc, double* out, cudaStream_t s);
// Mixed form: x += e, (rh, rl) -= L e in double-float, out[0] = rh.rh
// (r_lo of launch_lap_defect starts the pair)
void launch_lap_update_df(const Dims& d, double* x, const float* e, float* rh, float* rl, RedScratch sc, double* out,
                          cudaStream_t s);
// The mixed form's FP64-state defects evaluated with int64 block arithmetic
// and float pairs (no FP64 instruction; see dfloat.cuh). The Laplacian form
// needs n a power of two and returns false (nothing launched) otherwise.
bool launch_lap_defect_bfp(const Dims& d, float* r, const double* x, const double* b, RedScratch sc, double* out,
                           cudaStream_t s);
void launch_helm_defect_bfp(const Dims& d, int comp, double scale, const double* x, const double* b, float* r,
                            RedScratch sc, double* out, cudaStream_t s);
// One red (color 0) or black (color 1) Gauss-Seidel half sweep; omega:
// over-relaxation x + omega (gs - x) on levels with nx >= 64 (1 below).
// rev (here and in the residual, transfer and Jacobi launchers): blocks in
// reverse order (block_at, common.cuh) on the batched power-of-two kernels.
template <typename T>
void launch_rbgs(const Dims& d, int color, T* x, const T* b, cudaStream_t s, double omega = 1.0, int rev = 0);
// The red colour of a sweep from x = 0 (x's contents ignored, both colours
// written): the same bits as zeroing x and launch_rbgs(color 0).
template <typename T>
void launch_rbgs_from_zero(const Dims& d, T* x, const T* b, cudaStream_t s, double omega = 1.0, int rev = 0);
// One full red+black sweep per launch, out of place (xin -> xout), z-marching
// blocks fed by bulk asynchronous row copies; equals the two per-colour
// launches cell for cell. FY == 0: level not eligible (small, 2D, or rows not
// 16-byte multiples). err[0] |= 1 when a block gave up waiting for a copy.
struct PipeCfg {
    int FY = 0, ZC = 0, D = 0, grid = 0;
    size_t smem = 0;
};
template <typename T>
PipeCfg rbgs_pipe_cfg(const Dims& d);

// The V-cycle from level 0 of these levels down (smooth nu1, residual,
// restrict, ..., the one-block CG on the last level, prolong-add, smooth nu2)
// in one block: for the coarse levels (a few thousand cells or fewer), where
// launches cost more than work. Equals the launch-by-launch V-cycle bit for
// bit. For T = float the last level is solved in FP64 through cx64/cb64/cr64.
constexpr int kMaxTailLevels = 8;
template <typename T>
struct TailLevels {
    int nlev, nu1, nu2, maxit;
    Dims d[kMaxTailLevels];
    T* x[kMaxTailLevels];
    T* b[kMaxTailLevels];
    T* r[kMaxTailLevels];
    double *cx64, *cb64, *cr64, *cw_p, *cw_q;
    double tol;
    int* status;
};
template <typename T>
void launch_vcycle_tail(const TailLevels<T>& a, cudaStream_t s, int cluster = 1);
// Largest thread-block cluster (16, 8 or 4 CTAs) the cluster form of the
// V-cycle tail can be launched with on this device; 1: none.
int vcycle_tail_cluster_max();
template <typename T>
void launch_rbgs_pipe(const Dims& d, const PipeCfg& c, const T* xin, T* xout, const T* b, int* err, cudaStream_t s);
// Full-weighting restriction, src/mg/solver.h:153-181 (d = fine dims); zero
// (optional): the coarse iterate, set to zero in the same pass.
template <typename T>
void launch_restrict(const Dims& d, T* coarse, const T* fine, cudaStream_t s, int rev = 0, T* zero = nullptr);
// fine += P coarse (trilinear), src/mg/solver.h:71-151 and :211-212.
template <typename T>
void launch_prolong_add(const Dims& d, T* fine, const T* coarse, cudaStream_t s, int rev = 0);
// coarse_b = restriction of (b - L x), coarse_x = 0, in one pass (the
// residual stays in shared memory), for the levels resid_restrict_fused_ok
// takes: by default FP32 3D power-of-two levels with nx >= 256 (the column
// kernel); AFMIB_RESID_RESTRICT=1 the ring kernel, =0 none
bool resid_restrict_fused_ok(const Dims& d, size_t elem, const void* x, const void* b, const void* cb,
                             const void* cx);
// shared-memory opt-ins of the multigrid kernels (once per device, before
// any launch or stream capture)
void mg_kernel_attributes();
template <typename T>
void launch_resid_restrict(const Dims& d, T* coarse_b, T* coarse_x, const T* x, const T* b, cudaStream_t s,
                           int rev = 0);
// Prolongation that assigns (for the op-level API).
template <typename T>
void launch_prolong_assign(const Dims& d, T* fine, const T* coarse, cudaStream_t s);
// Coarsest-level solve (mean removal + CG on one block), src/mg/solver.h:264-271.
// status[0] receives 0 or 3 (not converged).
template <typename T>
void launch_coarse_solve(const Dims& d, T* x, T* b, T* r, T* p, T* q, double tol, int maxit, int* status,
                         cudaStream_t s);

}  // namespace afmib
