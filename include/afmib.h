/*
 * afmib — GB300 (sm_103a) immersed-boundary Navier–Stokes step, C ABI.
 *
 * The reference (best-of-both/afmibins) is a header-only C++14 template
 * library with no FFI: a caller instantiates ns::solver<G>, mg::solver<G>,
 * alg::conjugate_gradient, alg::div/grad and ib::grid::interpolate on
 * compile-time geometries. This header is the C boundary those calls are
 * rebuilt on; the C++ header shim under afmibins_gb300/src/{dt,alg,mg,ns,ib}
 * keeps the reference's template names and forwards to these entry points.
 * Each declaration cites the reference interface it replaces.
 *
 * Conventions
 *  - All field arrays are FP64, x fastest: i = x + nx*(y + ny*z).
 *  - u and w have nx*ny*nz entries. v has nx*(ny-1)*nz entries in channel
 *    mode (interior y faces, src/ib/mac_grid.h:75-105) and nx*ny*nz in
 *    periodic mode.
 *  - Wall vectors (channel mode) have nx*nz entries.
 *  - nz = 1 (periodic bc only) is a 2D grid in (x, y): the reference has no
 *    2D mode; every operator is its 3D row with the one-cell z extent folded
 *    into the diagonal (src/mg/laplacian.h:62-73), multigrid coarsens x and y,
 *    w stays zero, and the marker kernel is phi_x phi_y (spreading scale n^2,
 *    a marker's volume is its area measure; interpolation weight h^2).
 *  - Marker positions are X[M][3]; per-marker forces are F[3][M].
 *  - Pointers may be host or device memory (unified addressing); calls that
 *    return data to the host synchronise the solver's stream first.
 *  - Every call returns an afmib status; a non-zero status leaves a message
 *    in afmib_last_error(). Iterative solves are bounded and report
 *    AFMIB_ERR_NOCONV instead of looping (the reference loops forever,
 *    src/alg/cg.h:42, src/mg/solver.h:228).
 */
#ifndef AFMIB_H
#define AFMIB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct afmib_solver afmib_solver;

enum afmib_status {
    AFMIB_OK = 0,
    AFMIB_ERR_ARG = 1,      /* invalid argument or unsupported shape */
    AFMIB_ERR_CUDA = 2,     /* CUDA runtime error */
    AFMIB_ERR_NOCONV = 3,   /* iteration cap reached before the tolerance */
    AFMIB_ERR_BOUNDS = 4,   /* a marker within 2.5h of a channel wall */
    AFMIB_ERR_NAN = 5,      /* non-finite residual or marker position */
    AFMIB_ERR_STATE = 6,    /* call out of order (e.g. no markers set) */
    AFMIB_ERR_CAPACITY = 7  /* a fixed capacity exceeded (the no-allocation solve's array) */
};

enum { AFMIB_BC_PERIODIC = 0, AFMIB_BC_CHANNEL = 1 };
enum { AFMIB_FP64 = 0, AFMIB_MIXED = 1 };

typedef struct afmib_config {
    int nx, ny, nz;     /* cells (the reference's geometry<L,W,H,D>::nx, ny, nz); nz = 1: 2D */
    int n;              /* cells per unit length, 0 -> nx (geometry::n) */
    int bc;             /* AFMIB_BC_CHANNEL: the reference's walls in y; AFMIB_BC_PERIODIC */
    int precision;      /* AFMIB_FP64 (drop-in) or AFMIB_MIXED (FP32 inner, FP64 outer) */
    int mg_levels;      /* coarsenings of the pressure multigrid; 0 -> until a dimension is odd */
    int nu1, nu2;       /* smoothing sweeps of the FP64 V-cycles, 0 -> 2 (src/ns/projection.h:44);
                           the mixed form's FP32 inner cycles run their own V(2,1)
                           with red-black over-relaxation 1.25 on levels >= 64 */
    double mu, rho, dt; /* ns::solver(mu, rho, k, tol, ...), src/ns/solver.h:61-72 */
    double tol;         /* CG stops at ||r||_2 <= tol, MG at RMS(r) <= tol */
    int max_cg_iters;   /* 0 -> 1000 */
    int max_mg_cycles;  /* 0 -> 200 */
    double k_spring;    /* linear spring stiffness of the membrane */
    double inner_tol;   /* mixed precision: relative reduction per FP32 inner solve, 0 -> 1e-5 */
    int ib_fp32;        /* mixed precision: bit 0 spreads, bit 1 interpolates in FP32 (0: both FP64, the
                           default, which keeps the velocity within 1e-8 of the FP64 form) */
    int proj_start;     /* initial pressure of each projection: AFMIB_START_DEFAULT (FP64: from zero, the
                           reference's nested iteration, src/mg/solver.h:201-216; mixed: warm),
                           AFMIB_START_ZERO, or AFMIB_START_WARM (the previous pressure of the same
                           sub-step kind, BE or CN) */
    int walls_corrected; /* channel wall-velocity update after each projection: 0 the reference's
                           (src/ns/projection.h:86-104, its loop over nx*ny entries and its w rows
                           reading the x-gradient), 1 corrected (all nx*nz entries, w rows from the
                           z-gradient) */
    double k_bend;      /* bending stiffness of the membrane: force -k_bend L (L X) of the energy
                           k_bend/2 sum_i |(L X)_i|^2, L the graph Laplacian of the spring lists
                           (0: springs only; the reference has no membrane mechanics) */
} afmib_config;

enum { AFMIB_START_DEFAULT = 0, AFMIB_START_ZERO = 1, AFMIB_START_WARM = 2 };

typedef struct afmib_stats {
    long long substeps;   /* ns sub-steps taken (BE and CN each count one) */
    long long ib_steps;
    long long cg_iters;   /* total CG iterations */
    long long mg_cycles;  /* total V-cycles */
    long long outer_iters;/* mixed precision: FP64 defect-correction iterations */
    double last_mg_rms;   /* RMS residual at the end of the last pressure solve */
    double last_cg_norm;  /* ||r||_2 at the end of the last CG solve */
    int half;             /* 1 when the next sub-step is the CN step */
    int spread_tiles;     /* active tiles of the last spreading */
    long long kernel_launches;
} afmib_stats;

/* Lifecycle. `stream` is a cudaStream_t (0 -> a stream owned by the solver).
 * Replaces the construction of ns::solver / projection / helmholtz matrices,
 * src/ns/solver.h:61-72, without the initial projection (afmib_project). */
int afmib_create(const afmib_config* cfg, void* stream, afmib_solver** out);
int afmib_destroy(afmib_solver* s);
const char* afmib_error_string(int status);
const char* afmib_last_error(const afmib_solver* s);
int afmib_get_stats(const afmib_solver* s, afmib_stats* out);
int afmib_synchronize(afmib_solver* s);

/* Velocity state: the reference keeps references to the caller's u0, v0, w0
 * (src/ns/solver.h:54-56, 83-85). */
int afmib_set_velocity(afmib_solver* s, const double* u, const double* v, const double* w);
/* Drop the projections' warm-start potentials (and the multigrid contraction
 * estimate): the next projections start as on a new solver. afmib_set_velocity
 * keeps them (they are only a first guess), so that a loop feeding the
 * velocity back every step keeps its warm starts. */
int afmib_reset_warm_start(afmib_solver* s);
int afmib_get_velocity(afmib_solver* s, double* u, double* v, double* w);
/* p = (I - s*Delta) phi, ns::solver::get_p, src/ns/solver.h:86 */
int afmib_get_pressure(afmib_solver* s, double* p);
/* Channel wall velocities ut, ub, wt, wb (nx*nz each), mutated by every
 * sub-step like the caller's vectors in ns::solver::step, src/ns/projection.h:75-122. */
int afmib_set_walls(afmib_solver* s, const double* ut, const double* ub, const double* wt, const double* wb);
int afmib_get_walls(afmib_solver* s, double* ut, double* ub, double* wt, double* wb);

/* Projection of the current velocity: ns::projection::project, src/ns/projection.h:60-73
 * (called once by the ns::solver constructor, src/ns/solver.h:71). */
int afmib_project(afmib_solver* s);
/* One sub-step with the given face forces (null -> zero): the BE half step
 * and the CN step alternate like ns::solver::step, src/ns/solver.h:90-140. */
int afmib_ns_step(afmib_solver* s, const double* fx, const double* fy, const double* fz);

/* Lagrangian markers: positions X[M][3], spring neighbour lists in CSR form
 * (nstart[M+1], nidx[nstart[M]]), optional per-marker volumes (null -> 1).
 * Replaces ib::lagrangian_grid construction, src/ib/lagrangian_grid.h:50-55. */
int afmib_set_markers(afmib_solver* s, int M, const double* X, const int* nstart, const int* nidx, const double* vol);
int afmib_get_markers(afmib_solver* s, double* X);
/* Replace the positions of the current marker set (same M, same springs);
 * enqueued on the solver's stream without a host synchronisation. */
int afmib_set_marker_positions(afmib_solver* s, const double* X);
/* nsteps immersed-boundary steps: springs, spread, BE sub-step, two
 * interpolations with the midpoint marker update, spread, CN sub-step
 * (the coupling left as comments in test/ib_ns_test.cc:73-96). */
int afmib_ib_step(afmib_solver* s, int nsteps);

/* Snapshot of the solver state to a binary file (layout documented in
 * afmibins_gb300/csrc/snapshot_io.h; afmibins_gb300/snapshot.py reads it):
 * velocity (device layout, v with its wall plane), wall velocities and the
 * wall rows of the last pressure gradient, the pressure potential and its
 * warm-start copies, markers, springs and volumes,
 * the sub-step phase and the multigrid contraction estimate. Loading it into
 * a solver of the same grid and boundary conditions continues the run bit for
 * bit. The reference has no format (it prints with operator<<,
 * src/dt/vector.h:153-165). */
int afmib_save(afmib_solver* s, const char* path);
int afmib_load(afmib_solver* s, const char* path);

/* Spring stiffness k of the membrane (G_i = k * sum_j (X_j - X_i)). */
int afmib_set_spring(afmib_solver* s, double k);
/* Bending stiffness of the membrane (afmib_config.k_bend). */
int afmib_set_bending(afmib_solver* s, double kb);

/* ---- adjoint (no reference counterpart: the reference has no adjoint) ----
 * afmib_trajectory_forward runs nsteps IB steps from the current state and
 * keeps the state (u, X) every ckpt_every steps in device memory.
 * afmib_trajectory_adjoint takes the gradient of a loss with respect to the
 * final velocity (lam_u, lam_v, lam_w; null -> 0) and final markers
 * (lam_X[M][3]; null -> 0) and returns the gradients with respect to the
 * initial markers (grad_X0[M][3]), the stiffness k (*grad_k) and optionally
 * the initial velocity, recomputing each segment from its checkpoint.
 * Periodic domain, unit marker volumes and symmetric neighbour lists. */
int afmib_trajectory_forward(afmib_solver* s, int nsteps, int ckpt_every);
int afmib_trajectory_adjoint(afmib_solver* s, const double* lam_u, const double* lam_v, const double* lam_w,
                             const double* lam_X, double* grad_X0, double* grad_k, double* grad_u0, double* grad_v0,
                             double* grad_w0);

/* ---- single operators on caller buffers, on the solver's grid and stream ---- */
/* alg::div<nx,ny,nz,n>(d, u, v, w, top, bottom), src/alg/div.h:29-60 (top/bottom may be null) */
int afmib_div(afmib_solver* s, double* d, const double* u, const double* v, const double* w, const double* top,
              const double* bottom);
/* alg::grad<nx,ny,nz,n>(px, py, pz, p), src/alg/grad.h:29-44 */
int afmib_grad(afmib_solver* s, double* px, double* py, double* pz, const double* p);
/* ns::solver::advection, src/ns/solver.h:142-236 */
int afmib_advection(afmib_solver* s, double* ua, double* va, double* wa, const double* u, const double* v,
                    const double* w);
/* mg::solver<G>::solve(rhs): rhs is overwritten by the solution, returns the
 * V-cycle count in *cycles, src/mg/solver.h:218-237. A mixed-precision solver
 * solves by FP64 defect correction around FP32 V-cycles to the same RMS stop. */
int afmib_mg_solve(afmib_solver* s, double* rhs, int* cycles);
/* mg::solver::L * x, src/mg/laplacian.h:46-153 */
int afmib_lap_apply(afmib_solver* s, double* y, const double* x);
/* helmholtz_periodic / helmholtz_dirichlet (I + scale*Delta) * x,
 * src/ns/helmholtz.h:61-175, 218-319; comp 0/1/2 = u/v/w */
int afmib_helm_apply(afmib_solver* s, int comp, double scale, double* y, const double* x);
/* alg::conjugate_gradient(x, helmholtz(scale), b, tol), src/alg/cg.h:32-56 */
int afmib_helmholtz_cg(afmib_solver* s, int comp, double scale, double* x, const double* b, int* iters);
/* alg::smooth(x, L, b), src/alg/smooth.h:35-51: one Gauss-Seidel sweep of the
 * pressure Laplacian on x, here in red-black order (red cells, then black) */
int afmib_smooth(afmib_solver* s, double* x, const double* b);
/* Solver tolerance (the tol of ns::solver, mg::solver and conjugate_gradient) */
int afmib_set_tolerance(afmib_solver* s, double tol);
/* mg::solver::restriction / interpolation (assigning), src/mg/solver.h:153-181, 71-151 */
int afmib_restrict(afmib_solver* s, double* coarse, const double* fine);
int afmib_prolong(afmib_solver* s, double* fine, const double* coarse);
/* ib::grid::interpolate, spreading direction (mac_grid <- lagrangian_grid),
 * src/ib/grid.h:68-84: f = sum phi^3 * vol * F; F[3][M], vol may be null */
int afmib_spread(afmib_solver* s, int M, const double* X, const double* F, const double* vol, double* fx, double* fy,
                 double* fz);
/* ib::grid::interpolate, interpolation direction (lagrangian_grid <- mac_grid):
 * U[3][M] = sum phi^3 * h^3 * u */
int afmib_interp(afmib_solver* s, int M, const double* X, const double* u, const double* v, const double* w,
                 double* U);

/* Helmholtz CG that allocates nothing (no reference counterpart). For callers
 * that may not call cudaMalloc where they solve: code inside a memory pool or
 * arena that owns the process's device allocations, code under a strict
 * memory budget of its host framework, or inner loops that cannot take the
 * implicit synchronisation of an allocation. Same solve and stopping rule as
 * afmib_helmholtz_cg, on the caller's device buffers x (warm start, solution)
 * and b; its working vectors live in a file-scope device array (about
 * 6.5 MB) that every GPU holds once the library's device code is loaded on it,
 * until the process exits. Limits: nx*ny*nz <= 64^3 (larger ->
 * AFMIB_ERR_CAPACITY); 3D grids only (nx, ny, nz >= 2, else AFMIB_ERR_ARG);
 * periodic, or channel components 0 and 2. The first call on a device looks up
 * the array's address, which under CUDA's lazy module loading (the default)
 * also loads the device code and so reserves the array: make one warm-up call
 * (or set CUDA_MODULE_LOADING=EAGER) before the code that must not allocate,
 * and before any stream capture; later calls allocate nothing. Calls that
 * overlap on the GPU share the array and race. cudaDeviceReset while the
 * library is in use is not supported (the address is kept per device). */
int afmib_helmholtz_cg_noalloc(int nx, int ny, int nz, int n, int bc, int comp, double scale, double tol,
                               int max_iters, double* x, const double* b, int* iters, void* stream);

/* ---- per-kernel timing (no reference counterpart; the reference has no
 * profiling): while enabled, every kernel launch is bracketed by CUDA events
 * on the solver's stream and accumulated per kernel family with its
 * algorithmic bytes (each input array read once, each output written once). */
int afmib_profile_enable(afmib_solver* s, int on);
int afmib_profile_reset(afmib_solver* s);
int afmib_profile_count(const afmib_solver* s);
int afmib_profile_get(afmib_solver* s, int i, const char** name, long long* launches, double* ms, double* bytes);

#ifdef __cplusplus
}
#endif

#endif /* AFMIB_H */
