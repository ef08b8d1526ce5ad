/*
 * fishgpu.h -- C ABI of libfishgpu.so, a GB300 (sm_103a) structured-grid
 * Poisson solver for the fish.c / poissonfunctions.c path of bueler/p4pdes.
 *
 * Conventions
 *   - Every entry point returns an int status (FISHGPU_OK == 0).
 *   - Device arrays are explicit (`*_dev` or documented as device pointers);
 *     no hidden host<->device copies happen in the per-level call-backs.
 *     Only fishgpu_solve_host() takes host arrays.
 *   - Grid arrays are dense, x fastest: a[(k*my + j)*mx + i], indexed with
 *     GLOBAL (i,j,k) exactly like the DMDA arrays au/aF of the reference.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream); all work is stream-ordered.
 *   - No PETSc types appear: DMDALocalInfo, PoissonCtx and the PETSc option
 *     database are mirrored by fishgpu_info, fishgpu_ctx, fishgpu_opts.
 */
#ifndef FISHGPU_H_
#define FISHGPU_H_

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define FISHGPU_OK               0
#define FISHGPU_ERR_ARG          1  /* invalid argument / option value     */
#define FISHGPU_ERR_CUDA         2  /* CUDA runtime error                  */
#define FISHGPU_ERR_NOMEM        3  /* device allocation failed / budget   */
#define FISHGPU_ERR_NOT_CONVERGED 4 /* KSP diverged or reached max_it      */
#define FISHGPU_ERR_NONFINITE    5  /* NaN/Inf met during the solve        */
#define FISHGPU_ERR_TIMEOUT      6  /* a wait gave up (device or server)    */
#define FISHGPU_ERR_UNSUPPORTED  7  /* option the GPU library lacks        */
#define FISHGPU_ERR_NODEVICE     8  /* no CUDA device / wrong architecture */

/* ---- problem selection (replaces PoissonCtx's f_rhs/g_bdry pointers) -- */
enum { FISHGPU_MANUPOLY = 0, FISHGPU_MANUEXP = 1, FISHGPU_ZERO = 2, FISHGPU_USER = 3 };

/* Mirrors the DMDALocalInfo fields the call-backs use, plus the bounding box
   that the reference obtains with DMGetBoundingBox(info->da, ...)
   (c/ch6/poissonfunctions.c:34, :72). */
typedef struct {
  int dim;                 /* 1, 2, 3 */
  int mx, my, mz;          /* global nodes per direction (1 when unused) */
  int xs, ys, zs;          /* owned range start (global indices)        */
  int xm, ym, zm;          /* owned range size                          */
  double xmin[3], xmax[3]; /* bounding box                              */
} fishgpu_info;

/* Mirrors PoissonCtx (c/ch6/poissonfunctions.h:43-54).  The host function
   pointers f_rhs/g_bdry become a problem enum evaluated on the device, or,
   for FISHGPU_USER, device arrays holding f and g at every node. */
typedef struct {
  double Lx, Ly, Lz;
  double cx, cy, cz;
  int problem;             /* FISHGPU_MANUPOLY / MANUEXP / ZERO / USER   */
  int dim;                 /* selects the 1D/2D/3D manufactured formula  */
  const double *f;         /* FISHGPU_USER: device, f at every node      */
  const double *g;         /* FISHGPU_USER: device, g at every node      */
} fishgpu_ctx;

/* ---- drop-in DMDA local call-backs ------------------------------------ */

/* F = residual of -cx u_xx - cy u_yy - cz u_zz = f with Dirichlet rows, rows
   scaled by the cell volume; replaces Poisson1DFunctionLocal
   (c/ch6/poissonfunctions.c:4-26).  au, aF: device, whole grid. */
int Poisson1DFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                               const fishgpu_ctx *user, void *stream);
/* replaces Poisson2DFunctionLocal (c/ch6/poissonfunctions.c:29-65) */
int Poisson2DFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                               const fishgpu_ctx *user, void *stream);
/* replaces Poisson3DFunctionLocal (c/ch6/poissonfunctions.c:68-115) */
int Poisson3DFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF,
                               const fishgpu_ctx *user, void *stream);

/* q = J p with J the Jacobian the reference assembles (boundary rows:
   diagonal only; interior rows: boundary columns eliminated), applied
   matrix-free; optionally *pq_dot (device scalar) = p.q over the owned range.
   Replaces Poisson1DJacobianLocal + MatMult (c/ch6/poissonfunctions.c:117-150). */
int Poisson1DOperatorApply_gpu(const fishgpu_info *info, const double *p, double *q,
                               double *pq_dot, const fishgpu_ctx *user, void *stream);
/* replaces Poisson2DJacobianLocal + MatMult (c/ch6/poissonfunctions.c:152-193) */
int Poisson2DOperatorApply_gpu(const fishgpu_info *info, const double *p, double *q,
                               double *pq_dot, const fishgpu_ctx *user, void *stream);
/* replaces Poisson3DJacobianLocal + MatMult (c/ch6/poissonfunctions.c:195-258) */
int Poisson3DOperatorApply_gpu(const fishgpu_info *info, const double *p, double *q,
                               double *pq_dot, const fishgpu_ctx *user, void *stream);

/* Same result as Poisson{1,2,3}DOperatorApply_gpu (dimension from info->dim)
   for callers that may not allocate device memory once running (a serving
   loop working inside a fixed HBM budget, a host framework whose own pool owns
   the device): it allocates nothing and keeps the dot product's partial sums
   in a static device array of 4096 doubles + 256 B held by every GPU that
   loads the library.  Launches that would need more partial sums are rejected
   with FISHGPU_ERR_ARG.  All calls on a device share the array, so calls that
   overlap on the GPU race.  `stream` must belong to the current device (the
   array's address is that device's), else FISHGPU_ERR_ARG; the first call on
   a device may load the library's device code and should come before any
   stream capture.  This entry point has no counterpart in the reference. */
int PoissonOperatorApplyNoAlloc_gpu(const fishgpu_info *info, const double *p, double *q,
                                    double *pq_dot, const fishgpu_ctx *user, void *stream);

/* u = exact solution (= g) at every owned node; replaces Form{1,2,3}DUExact
   (c/ch6/fish.c:288-340); dimension taken from info->dim. */
int FormUExact_gpu(const fishgpu_info *info, double *u, const fishgpu_ctx *user, void *stream);

/* u = 0 (type 0) or uniform [0,1) noise from `seed` (type 1, the library's own
   generator), then u = g on the boundary when gbdry != 0; replaces
   InitialState (c/ch6/poissonfunctions.c:260-346). */
int InitialState_gpu(const fishgpu_info *info, int initial_type, int gbdry,
                     unsigned long long seed, double *u, const fishgpu_ctx *user, void *stream);

/* err_inf = max|u-uexact|, err_h = ||u-uexact||_2 / sqrt(prod(m-1)) over the
   whole grid; the report of c/ch6/fish.c:254-276.  Results to host doubles. */
int ErrorNorms_gpu(const fishgpu_info *info, const double *u, const fishgpu_ctx *user,
                   double *errinf, double *err2h, void *stream);

/* ---- fish options (mirror c/ch6/fish.c:154-185 plus the PETSc solver
        options fish's tests and studies use) ------------------------------ */
enum { FISHGPU_PC_NONE = 0, FISHGPU_PC_JACOBI = 1, FISHGPU_PC_MG = 2 };
enum { FISHGPU_SMOOTH_CHEBYSHEV = 0, FISHGPU_SMOOTH_RICHARDSON = 1 };
enum { FISHGPU_NORM_PRECONDITIONED = 0, FISHGPU_NORM_UNPRECONDITIONED = 1 };
enum { FISHGPU_FP64 = 0, FISHGPU_MIXED = 1 };
enum { FISHGPU_INITIAL_ZEROS = 0, FISHGPU_INITIAL_RANDOM = 1, FISHGPU_INITIAL_GIVEN = 2 };

typedef struct {
  fishgpu_ctx ctx;          /* -fsh_problem -fsh_cx.. -fsh_Lx.. -fsh_dim     */
  int mx, my, mz;           /* from -da_refine / -da_grid_{x,y,z}           */
  int da_refine;
  int initial_type;         /* -fsh_initial_type zeros|random (or GIVEN)    */
  int initial_gonboundary;  /* -fsh_initial_gonboundary                     */
  unsigned long long seed;  /* -fsh_seed (random initial iterate)           */
  double rtol, atol, dtol;  /* -ksp_rtol -ksp_atol -ksp_divtol              */
  int max_it;               /* -ksp_max_it                                  */
  int norm_type;            /* -ksp_norm_type preconditioned|unpreconditioned */
  int pc_type;              /* -pc_type mg|jacobi|none                      */
  int mg_levels;            /* -pc_mg_levels (0: da_refine+1)               */
  int mg_cycles;            /* -pc_mg_cycle_type v|w  (1|2)                 */
  int smooth_type;          /* -mg_levels_ksp_type chebyshev|richardson     */
  int smooth_its;           /* -mg_levels_ksp_max_it                        */
  double esteig[4];         /* -mg_levels_ksp_chebyshev_esteig a,b,c,d      */
  double richardson_scale;  /* -mg_levels_ksp_richardson_scale              */
  int precision;            /* -fsh_precision fp64|mixed                    */
  double inner_rtol;        /* -fsh_inner_rtol (mixed: FP32 inner floor)    */
  int inner_max_it;         /* -fsh_inner_max_it                            */
  int outer_max_it;         /* -fsh_outer_max_it                            */
  int graph_iters;          /* -fsh_graph_iters (CG iterations per graph)   */
  int monitor;              /* -ksp_monitor                                 */
  int converged_reason;     /* -ksp_converged_reason                        */
  int snes_monitor;         /* -snes_monitor[_short]                        */
  int fuse_smooth;          /* -fsh_fuse_smooth 0|1: the two post-smoothing
                               Chebyshev steps of a 3D FP32 level in one
                               temporally blocked kernel (default 0: slower
                               than two launches on GB300; the smoothed
                               iterate is bit-identical either way)        */
  int device_loop;          /* -fsh_device_loop 0|1: the CG loop as a
                               conditional graph node, one launch per inner
                               solve (default 1); 0 launches a graph of
                               graph_iters iterations per host read of the
                               stop flag (same kernels; profilers that skip
                               conditional bodies list every launch)        */
  int loop_cap;             /* -fsh_loop_cap: bodies (graph_iters CG
                               iterations each) the solve loop may run
                               before it gives up with FISHGPU_ERR_TIMEOUT
                               (0: max_it / graph_iters + 5, which a solve
                               that stops on its own never reaches)         */
  double first_floor_scale; /* -fsh_first_floor: mixed form, the first
                               refinement step's inner solve stops at
                               first_floor * kappa * pi h * 2^-24 (the FP32
                               floor of the accurate form; default 0.3)    */
  int inner_accurate;       /* -fsh_inner_accurate -1|0|1: mixed form, 1: the
                               inner FP32 CG applies J in difference form and
                               accumulates its solution in FP64, which moves
                               the FP32 floor of a refinement step from
                               ~kappa 2^-24 to ~kappa pi h 2^-24; 0: standard
                               FP32 apply and FP32 correction (8 fewer bytes
                               per node and iteration); -1 (default): 1 when
                               the standard form's two refinement steps
                               cannot reach rtol, that is when rtol <
                               0.3 kappa 2^-24 inner_rtol                  */
  int fuse_restrict;        /* -fsh_fuse_restrict 0|1: on 3D levels the
                               V-cycle's residual and its restriction run as
                               one kernel that keeps the fine residual in
                               shared memory (bit-identical to the
                               two-kernel form; default 0: measured slower,
                               0.51 ms against 0.27 + 0.12 ms at 513^3)    */
  int tma_apply;            /* -fsh_tma_apply 0|1: the accurate inner form's
                               CG direction update + apply on 3D grids reads
                               its planes from a shared-memory ring filled by
                               bulk tensor copies (default 0: measured level
                               with the slot march, 0.79 against 0.80 ms at
                               513^3, and the solve no faster)             */
  int vtail;                /* -fsh_vtail 0|1: the V-cycle's smallest levels
                               below the finest (up to 1200 nodes: 33^2,
                               9^3) run in one block per grid, a barrier
                               between phases instead of a launch (default
                               1; bit-identical to 0)                      */
  int vtail_points;         /* -fsh_vtail_points: largest level (nodes per
                               grid) the tail takes (0: the limits above)  */
  int persist;              /* -fsh_persist -1|0|1: each CG solve (its
                               set-up, iterations and V-cycles) as ONE
                               cooperative launch with a grid-wide barrier
                               between phases, for grids too small to fill
                               the GPU with a launch per phase (2D/3D, MG
                               with two Chebyshev steps, V-cycles, the
                               device loop); -1 (default): when the finest
                               grid has at most persist_points nodes      */
  int persist_points;       /* -fsh_persist_points: that limit (0: 2.5e6
                               for the FP64 form, 5e5 for the mixed
                               form)                                      */
  int persist_tail;         /* -fsh_persist_tail: largest level (nodes) the
                               persistent solve runs in its block 0 (0:
                               300 in FP64, 1200 in FP32)                  */
  int fuse_cgr;             /* -fsh_fuse_cgr 0|1: the mixed form's inner CG
                               iterations run their residual update
                               r -= alpha w inside the V-cycle's first
                               smoothing pass (one pass over r and w
                               instead of two, a second r buffer; MG with
                               two Chebyshev steps; default 1,
                               bit-identical to 0)                        */
  int coop_tail;            /* -fsh_coop_tail N: in launch-per-phase solves
                               of a single grid, the V-cycle's levels from
                               the largest of at most N nodes (below the
                               finest) down run as ONE cooperative launch,
                               a grid-wide barrier between phases (MG with
                               two Chebyshev steps, V-cycles; bit-identical
                               to 0).  0 (default): off, measured no faster
                               than the graphs' launches; -1:
                               FISHGPU_COOP_TAIL_POINTS                   */
  int pair_y;               /* -fsh_pair_y 0|1: the mixed form's accurate
                               inner CG updates its FP64 correction every
                               other iteration, two steps at a time
                               (default 1, bit-identical to 0)            */
} fishgpu_opts;

#define FISHGPU_COOP_TAIL_POINTS 300000

#define FISHGPU_MAX_HIST 512
#define FISHGPU_MAX_OUTER 32

typedef struct {
  int its;                  /* KSP iterations (mixed: inner, summed)        */
  int reason;               /* PETSc KSPConvergedReason numbering           */
  int outer_its;            /* mixed: refinement steps                      */
  int nhist;                /* residual-norm history entries               */
  double hist[FISHGPU_MAX_HIST];
  double fnorm0, fnorm1;    /* ||F(u0)||_2, ||F(u)||_2                      */
  double errinf, err2h;     /* vs the exact solution (manupoly/manuexp/zero) */
  double true_rel_resid;    /* ||b - J y||_2 / ||b||_2 of the linear solve  */
  double setup_ms, solve_ms;/* device time, CUDA events                     */
  long long dofs;           /* mx*my*mz                                     */
  long long launches;       /* kernels of this library launched by the solve */
  int inner_its[FISHGPU_MAX_OUTER]; /* mixed: inner CG iterations per refinement step */
} fishgpu_report;

const char *fishgpu_strerror(int code);
/* PETSc-style reason name, e.g. "CONVERGED_RTOL" */
const char *fishgpu_reason_name(int reason);

/* defaults of fish.c + PETSc, except pc_type defaults to mg (PETSc's
   one-rank default ILU is sequential and not offered by this library) */
int fishgpu_opts_default(fishgpu_opts *o);
/* parse fish's flag spellings; unknown flags are ignored as PETSc does */
int fishgpu_opts_parse(fishgpu_opts *o, int argc, const char *const *argv);

/* ---- solver: device-resident hierarchy --------------------------------- */
typedef struct fishgpu_solver_s fishgpu_solver;

int fishgpu_solver_create(const fishgpu_opts *o, void *stream, fishgpu_solver **out);
/* Full fish flow (c/ch6/fish.c:237-280 with SNESKSPONLY): u0 from the
   options (or u_dev itself for FISHGPU_INITIAL_GIVEN), F(u0), KSP solve of
   J y = F(u0), u = u0 - y, errors.  u_dev: device, mx*my*mz doubles. */
int fishgpu_solver_solve(fishgpu_solver *s, double *u_dev, fishgpu_report *rep);
int fishgpu_solver_destroy(fishgpu_solver *s);
/* device bytes held by the solver */
long long fishgpu_solver_bytes(const fishgpu_solver *s);

/* Same flow with HOST arrays on an existing solver (the end-to-end form):
   for FISHGPU_USER solvers created with ctx.f == ctx.g == NULL the solver owns
   device copies of f and g, and f_host/g_host (mx*my*mz doubles each) are
   copied in first; u_host receives the solution (and supplies u0 for
   FISHGPU_INITIAL_GIVEN).  All copies are stream-ordered on the solver's
   stream and included in rep->solve_ms. */
int fishgpu_solver_solve_host(fishgpu_solver *s, const double *f_host, const double *g_host,
                              double *u_host, fishgpu_report *rep);

/* n host-array solves in order (FISHGPU_USER), each as fishgpu_solver_solve_host
   would do it (g_host NULL, or g_host[k] NULL: zero boundary data), pipelined:
   while problem k is solved, f_host[k+1] is copied in and u_host[k-1] out on
   two copy streams through device staging buffers (2 more dense arrays,
   allocated at the first call).  Pinned f_host and u_host let the copies
   overlap the solves.  reps[k]: problem k's report (solve_ms: its solve). */
int fishgpu_solver_solve_host_many(fishgpu_solver *s, int n, const double *const *f_host,
                                   const double *const *g_host, double *const *u_host,
                                   fishgpu_report *reps);

/* host -> device bytes fishgpu_solver_solve_host moves for f and g (FISHGPU_USER):
   all of f; all of g, or only its boundary nodes when g_host is pinned memory
   (the solver reads g nowhere else) */
long long fishgpu_solver_host_bytes_in(const fishgpu_solver *s, const double *g_host);

/* device bytes fishgpu_solver_create would allocate (plus the host-array
   buffers of fishgpu_solver_solve_host for FISHGPU_USER); -1 if invalid */
long long fishgpu_solver_estimate_bytes(const fishgpu_opts *o);

/* one-shot create + solve + destroy */
int fishgpu_solve(const fishgpu_opts *o, double *u_dev, fishgpu_report *rep);

/* End-to-end form with HOST arrays: copies f_host and g_host (FISHGPU_USER
   data, may be NULL for the built-in problems) to the device, solves, copies
   the solution to u_host.  The copies are stream-ordered on the solver's
   stream and included in rep->solve_ms. */
int fishgpu_solve_host(const fishgpu_opts *o, const double *f_host, const double *g_host,
                       double *u_host, fishgpu_report *rep);

/* Times `reps` launches of one solver kernel on the finest level with the
   solver's resident data (CUDA events on the solver's stream).  Names:
   "smooth", "smooth_first", "smooth_dots", "smooth_zero", "post2", "cgp_apply",
   "cgp_apply_acc" (mixed form: the accurate inner form's apply), "cgp_apply_acc_pair" (the two
   launches the solve alternates: y64 left alone, then both owed updates; one rep is the pair),
   "cgp_apply_tma" (the same from the
   TMA ring, 3D), "cg_update", "resid_restrict" (3D), "grid_sync" (one grid-wide barrier of the
   persistent solve; bytes 0), "demote" (mixed form: an inner solve's set-up from the FP64 residual),
   "resid", "apply", "restrict", "prolong", "residual64".  Reports the mean ms
   per launch and the algorithmic bytes one launch moves. */
int fishgpu_solver_time_kernel(fishgpu_solver *s, const char *name, int reps,
                               double *ms_per_launch, double *bytes_per_launch);

/* Self-test of the persistent solve's grid barrier and its time limit: one
   barrier over the solve's blocks, with block 0 leaving without arriving
   when `missing` is nonzero.  Returns FISHGPU_ERR_TIMEOUT when the other
   blocks' bounded waits ran out (expected with missing, after ~0.2 s),
   FISHGPU_OK when the barrier completed; FISHGPU_ERR_UNSUPPORTED when the
   solver has no persistent solve.  The device stays usable either way. */
int fishgpu_solver_barrier_selftest(fishgpu_solver *s, int missing);

/* Measures the current device's FP64 FMA throughput in TFLOP/s (an FMA is 2
   flops): `reps` timed launches of a kernel of independent FMA chains on
   every SM, after one warm-up launch; the best launch counts.  The
   denominator for the FP64-bound kernels (the FP64 residual). */
int fishgpu_fp64_fma_rate(int reps, double *tflops);

/* ---- batches: many independent 2D problems of uneven sizes -------------
   -Laplace(u) = f on the unit square, u = 0 on the boundary, fish's 5-point
   discretisation (cx = cy = 1), n x n nodes with n = 2^k + 1.  Solved with
   the mixed form (FP64 refinement around FP32 CG + FP32 V-cycle, levels down
   to 3 x 3).  Instances of one size run together: one launch per multigrid
   phase covers all of them; size groups run concurrently. */
typedef struct {
  double rtol, atol;      /* on the FP64 true residual, per instance      */
  double inner_rtol;      /* FP32 inner CG floor                          */
  int inner_max_it;       /* per refinement step                          */
  int outer_max_it;
  int smooth_its;         /* Chebyshev/Jacobi steps per level (2: V(2,2)) */
  int mg_cycles;          /* 1 = V, 2 = W                                 */
  double esteig[4];
  int tune;               /* pick each level's tiles (block size, rows per
                             thread) by timing one smoothing step          */
  int inner_accurate;     /* as fishgpu_opts.inner_accurate, per size group (default -1) */
  int tune_sweeps;        /* with tune: smoothing steps per level of each
                             size group (1, 2 or 3) picked by timing batched
                             solves of up to 32 of its instances (default 1;
                             0: smooth_its for every group)              */
} fishgpu_batch_opts;

typedef struct {
  int ninst, groups, converged, max_outer, max_inner;
  long long total_inner_its, dofs, launches;
  double solve_ms;
} fishgpu_batch_report;

typedef struct fishgpu_batch_s fishgpu_batch;

int fishgpu_batch_opts_default(fishgpu_batch_opts *o);
/* n[q]: nodes per side of instance q (2^k + 1); allocates every hierarchy */
int fishgpu_batch_create(const fishgpu_batch_opts *o, int ninst, const int *n, fishgpu_batch **out);
/* f[q], u[q]: device pointers to dense n[q] x n[q] arrays (x fastest) */
int fishgpu_batch_solve(fishgpu_batch *b, const double *const *f, double *const *u, fishgpu_batch_report *rep);
/* per size group g (largest first): nodes per side, instances and the
   smoothing steps per level in use; returns the number of groups */
int fishgpu_batch_groups(const fishgpu_batch *b, int *n, int *count, int *sweeps);
/* per-instance results of the last solve (host arrays of ninst, any may be NULL) */
int fishgpu_batch_results(const fishgpu_batch *b, int *inner_its, int *outer_its, double *rel_resid, int *reason);
int fishgpu_batch_destroy(fishgpu_batch *b);

/* ---- same-size groups: `count` n x n instances solved together ----------
   One size group of a batch on its own stream (no device-wide
   synchronisation): the server's unit of merged 2D requests.  A solve takes
   k <= count host arrays (n*n doubles each); instances k .. count-1 are
   empty (f = 0: converged at once, their planes skip every kernel).  Every
   instance's result is independent of the others and of count (per-plane
   reductions, fixed tiles with o->tune = 0): bit-identical to the same
   instance in a group of one. */
typedef struct fishgpu_group_s fishgpu_group;
int fishgpu_group_create(const fishgpu_batch_opts *o, int n, int count, fishgpu_group **out);
long long fishgpu_group_bytes(const fishgpu_group *g);
/* per instance q < k: inner (summed) and outer iterations, FP64 true
   relative residual; returns the solve's status */
int fishgpu_group_solve_host(fishgpu_group *g, int k, const double *const *f_host, double *const *u_host, int *its,
                             int *outer_its, double *rel_resid);
int fishgpu_group_destroy(fishgpu_group *g);

/* ---- server: continuous batching of independent solves ----------------
   Each request is -Laplace(u) = f (fish's operator, cx = cy = cz = 1) on the
   unit square/cube with u = 0 on the boundary, n nodes per side (2^k + 1),
   f and u host arrays (n^dim doubles, x fastest) that stay valid until the
   request is waited for.  A request starts as soon as a worker is free and
   a solver for its size fits in the HBM budget; solvers stay device-resident
   in a pool keyed by size (idle ones of other sizes are evicted LRU-first
   when room is needed).  Workers run on their own streams, so solves
   overlap on the device. */
typedef struct {
  long long hbm_budget_bytes; /* device bytes the pooled solvers may hold    */
  int workers;                /* concurrent solves                           */
  double rtol;                /* true relative residual per request          */
  int precision;              /* FISHGPU_MIXED (default) or FISHGPU_FP64     */
  int fifo;                   /* 1: a request waits for every earlier one    */
  int batch_max;              /* mixed form: 2D requests of one size queued
                                 together are merged, up to batch_max, into
                                 one group solve
                                 (fishgpu_group; groups of 1, 2, 4, ... up to
                                 batch_max instances are pooled); 1: every
                                 request its own solver (default 16)        */
} fishgpu_server_opts;

typedef struct {
  int status;                 /* library status of the solve                */
  int its, outer_its;
  double rel_resid;
  double queue_ms, service_ms, latency_ms; /* host clock, submit -> done    */
} fishgpu_server_result;

typedef struct fishgpu_server_s fishgpu_server;

int fishgpu_server_opts_default(fishgpu_server_opts *o);
int fishgpu_server_create(const fishgpu_server_opts *o, fishgpu_server **out);
int fishgpu_server_submit(fishgpu_server *s, int dim, int n, const double *f_host, double *u_host,
                          long long *ticket);
/* timeout_ms < 0: wait without limit; FISHGPU_ERR_TIMEOUT when not finished */
int fishgpu_server_wait(fishgpu_server *s, long long ticket, double timeout_ms, fishgpu_server_result *res);
int fishgpu_server_stats(fishgpu_server *s, long long *pooled_bytes, int *pooled_solvers, long long *created,
                         long long *evicted);
/* group solves run and the requests they served */
int fishgpu_server_group_stats(fishgpu_server *s, long long *group_solves, long long *grouped_requests);
int fishgpu_server_destroy(fishgpu_server *s);

/* ---- minimal-surface equation (c/ch7/minimal.c) -------------------------
   -div( (1 + |grad u|^2)^q grad u ) = 0 on the unit square, u = g on the
   boundary (catenoid or tent data, minimal.c:27-42), 9-point finite
   differences (FormFunctionLocal, minimal.c:210-282).  Newton (PETSc
   SNESNEWTONLS with the cubic backtracking line search, SNESConvergedDefault)
   with the exact Jacobian applied matrix-free; each Newton step J Y = F is
   solved by FP32 BiCGStab right-preconditioned with the FP32 Poisson
   multigrid V-cycle (the preconditioning matrix of minimal.c:142-145), while
   F(u), the norms, the line search and the update stay FP64. */
#define FISHGPU_MS_TENT     0
#define FISHGPU_MS_CATENOID 1
/* The same Newton solver serves the Liouville-Bratu equation of
   c/ch7/solns/bratu2D.c, -Laplace(u) - lambda e^u = 0 (model FISHGPU_NL_BRATU,
   5-point residual bratu2D.c:188-217, u = 0 or Liouville's exact solution on
   the boundary, initial iterate 0). */
#define FISHGPU_NL_MINIMAL       0
#define FISHGPU_NL_BRATU         1
/* ... and the obstacle problem of c/ch12/obstacle.c (model FISHGPU_NL_OBSTACLE):
   -Laplace(u) = 0 on (-2,2)^2, u >= psi (hemisphere with a skirt), g = the
   exact solution, Poisson2DFunctionLocal as residual; the variational
   inequality is solved by the reduced-space active-set Newton method (PETSc
   SNESVINEWTONRSLS semantics: projection onto the bounds, active set
   u <= psi + 1e-8 with F > 0, Newton on the inactive set, residual norm over
   the inactive set). */
#define FISHGPU_NL_OBSTACLE      2
#define FISHGPU_BRATU_ZERO       0
#define FISHGPU_BRATU_LIOUVILLE  1

typedef struct {          /* MinimalCtx / BratuCtx + the boundary function   */
  int problem;            /* minimal: TENT / CATENOID; Bratu: ZERO / LIOUVILLE */
  double q;               /* exponent (default -1/2)                        */
  double catenoid_c;      /* catenoid parameter, >= 1 (default 1.1)         */
  double tent_H;          /* tent door height (default 1)                   */
  int model;              /* FISHGPU_NL_MINIMAL (default) / FISHGPU_NL_BRATU */
  double lambda;          /* Bratu: coefficient of e^u (default 1)          */
} fishgpu_ms_ctx;

typedef struct {
  fishgpu_ms_ctx ctx;
  int mx, my;             /* first grid: 3x3 refined -da_refine times        */
  int grid_sequence;      /* -snes_grid_sequence: further refinements        */
  int exact_init;         /* -ms_exact_init (catenoid, q = -1/2)             */
  double rtol, atol, stol;/* -snes_rtol/atol/stol: 1e-8, 1e-50, 1e-8         */
  int max_it;             /* -snes_max_it: 50                                */
  int line_search;        /* 1: bt (default), 0: basic (full Newton steps)  */
  double ksp_rtol;        /* -ksp_rtol: 1e-5                                 */
  int ksp_max_it;         /* -ksp_max_it: 10000                              */
  int pc_type;            /* FISHGPU_PC_MG (default) or FISHGPU_PC_NONE      */
  int mg_levels;          /* 0: down to 3x3                                  */
  int monitor_degree;     /* -ms_monitor: quadrature degree 1..3, 0 = off    */
  int snes_monitor, converged_reason, ksp_converged_reason; /* driver flags  */
  int loop_cap;           /* -ms_loop_cap: bodies the inner BiCGStab loop may
                             run per Newton step before the solve gives up
                             with FISHGPU_ERR_TIMEOUT (0: ksp_max_it / iterations
                             per body + 5, never reached by a solve that stops) */
  int inner_block;        /* -ms_inner_block 0|1: on grids of up to 4096 nodes whose
                             preconditioner is one exact coarse solve, the whole
                             inner BiCGStab runs in one block (default 1)    */
  int inner_persist;      /* -ms_inner_persist N: on multigrid grids of up to N
                             nodes the whole inner BiCGStab solve runs as one
                             cooperative launch (0: never; default -1: the
                             measured limit, FISHGPU_MS_PERSIST_POINTS)       */
  int vtail_points;       /* -ms_vtail_points N: the Poisson V-cycle's levels of
                             at most N nodes run in one block (the coarsest
                             always; 0: the fish solver's default)           */
} fishgpu_ms_opts;

#define FISHGPU_MS_PERSIST_POINTS 600000

#define FISHGPU_MS_MAX_GRIDS 12
#define FISHGPU_MS_MAX_ITS   64

typedef struct {
  int ngrids;                                  /* grids solved (1 + grid_sequence) */
  int m[FISHGPU_MS_MAX_GRIDS];                 /* nodes per side of each grid      */
  int its[FISHGPU_MS_MAX_GRIDS];               /* Newton iterations                */
  int reason[FISHGPU_MS_MAX_GRIDS];            /* SNES converged reason            */
  int ksp_its[FISHGPU_MS_MAX_GRIDS][FISHGPU_MS_MAX_ITS]; /* inner iterations per step */
  int ksp_reason[FISHGPU_MS_MAX_GRIDS][FISHGPU_MS_MAX_ITS];
  double fnorm[FISHGPU_MS_MAX_GRIDS][FISHGPU_MS_MAX_ITS + 1];
  double area[FISHGPU_MS_MAX_GRIDS][FISHGPU_MS_MAX_ITS + 1][3]; /* area, Dmin, Dmax */
  double errinf;                               /* catenoid, q = -1/2; else -1      */
  double solve_ms;                             /* all grids, device time           */
  long long dofs;                              /* nodes of the last grid           */
  long long total_ksp_its;
  long long nfuncs;                            /* residual evaluations            */
  double grid_ms[FISHGPU_MS_MAX_GRIDS];        /* device time per grid            */
  double err1;                                 /* obstacle: mean |u - u_exact|    */
  double active_area_err;                      /* obstacle: |area(A) - pi a^2| / pi a^2 */
  long long n_active;                          /* obstacle: nodes of the active set */
  int inner_form[FISHGPU_MS_MAX_GRIDS];        /* how each grid's inner solves ran:
                                                  0 launch-per-phase graphs, 1 one
                                                  block, 2 one cooperative launch */
} fishgpu_ms_report;

int fishgpu_ms_opts_default(fishgpu_ms_opts *o);
int fishgpu_bratu_opts_default(fishgpu_ms_opts *o);  /* model Bratu, lambda 1, u = 0 on the boundary */
int fishgpu_obstacle_opts_default(fishgpu_ms_opts *o); /* model obstacle (c/ch12/obstacle.c defaults) */
/* minimal.c's options (-ms_*, -da_refine, -da_grid_x/y, -snes_*, -ksp_rtol,
   -ksp_max_it, -pc_type mg|none, -snes_linesearch_type bt|basic, and bratu2D.c's
   -lb_lambda, -lb_exact, -lb_showcounts); options of
   PETSc's Jacobian handling (-snes_fd_color, -snes_mf_operator,
   -mat_is_symmetric) are accepted: the Jacobian is always the exact one */
int fishgpu_ms_opts_parse(fishgpu_ms_opts *o, int argc, const char *const *argv);
const char *fishgpu_snes_reason_name(int reason);

typedef struct fishgpu_ms_solver_s fishgpu_ms_solver;
/* set-up of every grid (hierarchies, buffers, graphs); stream NULL: own */
int fishgpu_ms_solver_create(const fishgpu_ms_opts *o, void *stream, fishgpu_ms_solver **out);
/* one solve from the initial iterate; u_host (last grid, mx*my doubles, x
   fastest) may be NULL */
int fishgpu_ms_solver_solve(fishgpu_ms_solver *s, double *u_host, fishgpu_ms_report *rep);
int fishgpu_ms_solver_destroy(fishgpu_ms_solver *s);
int fishgpu_ms_solve(const fishgpu_ms_opts *o, double *u_host, fishgpu_ms_report *rep);

/* Drop-in residual call-back: FormFunctionLocal, c/ch7/minimal.c:210-282;
   info->dim must be 2, whole-grid device arrays, global (i,j) indexing */
int MinimalFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF, const fishgpu_ms_ctx *ctx,
                             void *stream);
/* FormFunctionLocal of c/ch7/solns/bratu2D.c:188-217 (liouville: g of :62-68) */
int BratuFunctionLocal_gpu(const fishgpu_info *info, const double *au, double *aF, double lambda, int liouville,
                           void *stream);

/* ---- PETSc binary files (host arrays) ----------------------------------
   The format of PETSc's binary viewer (VecView/MatView, VecLoad/MatLoad;
   c/ch12/obstacle.c:138-144, c/ch2/loadsolve.c): big-endian; a Vec is
   classid 1211214, n, n doubles; an AIJ Mat is classid 1211216, M, N, nz,
   row lengths, column indices, values.  `index` counts objects in the file. */
int fishgpu_petsc_vec_write(const char *path, int append, const double *x, long long n);
int fishgpu_petsc_vec_read(const char *path, int index, double *x, long long cap, long long *n);
int fishgpu_petsc_mat_write_aij(const char *path, int append, int M, int N, const long long *rowptr,
                                const int *col, const double *val);
int fishgpu_petsc_mat_read_aij(const char *path, int index, int *M, int *N, long long *nz, long long *rowptr,
                               int *col, double *val);

#ifdef __cplusplus
}
#endif
#endif
