/*
 * vfs_gpu.h -- C ABI of the GB300 pressure-projection step of VFS.
 *
 * Drop-in for the reference's pressure path (trunglendsu/VFS_v3p2):
 *   PoissonLHSNew   poisson.c:976-1691        -> vfs_poisson_lhs
 *   PoissonRHS      poisson_hypre.c:272-477,
 *                   poisson.c:1789-1915        -> vfs_poisson_rhs
 *   PoissonSolver_MG mhv_poisson.c:2121-2359,
 *   PoissonSolver_Hypre poisson_hypre.c:580-771 -> vfs_poisson_solve
 *   UpdatePressure  poisson.c:2473-2632       -> vfs_update_pressure
 *   Projection      poisson.c:2122-2470       -> vfs_projection
 *   Divergence      main.c:1244-1390          -> vfs_divergence_max
 *   Flow_Solver pressure section, solvers.c:871-931 -> vfs_projection_step
 *
 * Plain C: no PETSc, HYPRE or CUDA types.  Every function returns an int
 * status (VFS_OK = 0); vfs_last_error() gives the message of the last failure
 * on a context.  Host buffers are borrowed for the duration of a call.
 * Fields use the reference's DMDA array layout: extents mx = ni + 2,
 * my = nj + 2, mz = nk + 2 (one ghost/boundary cell per side), element
 * (i, j, k) at ((k * my) + j) * mx + i; vector fields (Cmpnts: node
 * coordinates, Ucont, Ucat) are 3 doubles per element.
 *
 * The device state of a grid (metrics, operator, multigrid hierarchy,
 * Ucont, p, phi, Krylov basis) belongs to the context and stays resident in
 * HBM between calls.  A context is used by one host thread at a time.
 */
#ifndef VFS_GPU_H
#define VFS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define VFS_OK 0
#define VFS_ERR_ARG 1      /* invalid argument or unsupported grid */
#define VFS_ERR_CUDA 2     /* CUDA runtime error */
#define VFS_ERR_NOMEM 3    /* HBM budget exceeded or allocation failure */
#define VFS_ERR_NOTCONV 4  /* solver stopped at maxit above rtol */
#define VFS_ERR_STATE 5    /* call order (e.g. solve before the LHS) */
#define VFS_ERR_NUMERIC 6  /* NaN or Inf in the right-hand side or iterates */
#define VFS_ERR_BUSY 7     /* serving: no free slot or memory right now */
#define VFS_ERR_IO 8       /* file missing, unreadable, truncated or not a PETSc Vec */

#define VFS_FP64 0   /* plain: FP64 multigrid inside FP64 FGMRES */
#define VFS_MIXED 1  /* FP32 multigrid (FP32 coefficients) inside FP64 FGMRES */
#define VFS_ORTH_CGS 1
#define VFS_ORTH_CGS2 2

/* Fields for vfs_set_field / vfs_get_field. */
#define VFS_FIELD_UCONT 0  /* 3 doubles per cell (AoS), contravariant flux */
#define VFS_FIELD_P 1      /* pressure */
#define VFS_FIELD_PHI 2    /* pressure correction (solution) */
#define VFS_FIELD_RHS 3    /* Poisson right-hand side */
#define VFS_FIELD_UCAT 4   /* 3 doubles per cell (AoS), Cartesian velocity */
#define VFS_FIELD_NVERT 5  /* immersed-boundary mask */
#define VFS_FIELD_USTAR 6  /* 3 doubles per cell (AoS), resident intermediate flux */

typedef struct vfs_ctx vfs_ctx;

typedef struct {
  int device;                           /* CUDA device ordinal */
  unsigned long long hbm_budget_bytes;  /* 0 = no limit; grids beyond it are refused */
  int max_inflight;                     /* serving: requests in flight at once (0 = 16) */
} vfs_config;

typedef struct {
  int mx, my, mz;                       /* ghosted extents ni+2, nj+2, nk+2 */
  int i_periodic, j_periodic, k_periodic;
  int mg_levels;                        /* levels including the finest (>= 1) */
  int semi_i, semi_j, semi_k;           /* semi-coarsening per axis (-mg_*_semi) */
  int immersed;                         /* 0: no body, 1: IB flux balance (VolumeFlux) */
  const double* coor;                   /* host [mz][my][mx][3] node coordinates, nodes 0..n valid */
  const double* nvert;                  /* host [mz][my][mx] (0 fluid, 1 IB node, >1 solid) */
} vfs_grid_desc;

#define VFS_SMOOTH_JACOBI 0
#define VFS_SMOOTH_CHEBYSHEV 1

typedef struct {
  int precision;   /* VFS_FP64 or VFS_MIXED */
  double rtol;     /* relative tolerance on the aj-scaled residual (see div_tol) */
  int maxit;       /* maximum preconditioner applications */
  int restart;     /* FGMRES restart length (<= 64) */
  int nu1, nu2;    /* pre / post y-line smoothing sweeps per level */
  double omega;    /* line-Jacobi damping */
  int warm_start;  /* 1: start from the resident phi, 0: from zero */
  double div_tol;  /* > 0: also require max |div u| <= div_tol after the projection */
  int orth;        /* Gram-Schmidt of the Arnoldi step: VFS_ORTH_CGS (one
                      classical pass, the reference's PETSc GMRES default) or
                      VFS_ORTH_CGS2 (classical with one re-orthogonalisation) */
  int smooth_cols;  /* y-line smoother tile: i-columns per block, 0 (automatic: 32, fewer
                       for long lines), 8, 16 or 32 */
  int nu1_coarse, nu2_coarse;  /* sweeps on the levels below the finest (-1, the
                                  default: nu1 / nu2).  With the constant
                                  (Jacobi) damping, more coarse sweeps save
                                  iterations on one large grid (5 / 5 on
                                  256x128x128); the Chebyshev damping needs
                                  none beyond nu1 / nu2 */
  int mg_half;  /* VFS_MIXED only: storage of the multigrid levels' operator.
                   0 (the default): FP32 in face form, the row being aj times
                   the divergence of the cell's six face fluxes: per cell its
                   three faces' FP32 weights (g11, g22, g33 and the cross
                   weights with the one-sided regime folded in) and aj
                   carrying the i-k cross terms' regime code bits in its four
                   low mantissa bits (channel and sphere grids, whose only
                   cross terms are the i-k ones: a sweep streams 40 instead of
                   60 bytes per cell); on levels with i-j or j-k cross terms
                   (terrain) also the four other cross weights, each with its
                   own code in its two low mantissa bits (56 instead of 92
                   bytes per cell).  2: the assembled FP32 coefficients on
                   every level.  1: FP16 normalised by the
                   diagonal, with an FP16 centre-slot correction that keeps
                   every row sum.  The arithmetic is FP32 in every case, and
                   the FP64 FGMRES operator is the same. */
  int smoother;       /* VFS_SMOOTH_CHEBYSHEV (the default) or VFS_SMOOTH_JACOBI.
                         Both are y-line Jacobi sweeps x += w T^-1 (b - A x), T
                         the j-tridiagonal part of A.  JACOBI: w = omega on every
                         sweep.  CHEBYSHEV: a level's n pre-sweeps take w_k =
                         1 / theta_k, theta_k (k = 1..n, descending) the roots of
                         the degree-n Chebyshev polynomial on [cheb_hi /
                         cheb_ratio, cheb_hi], and its post-sweeps the same in
                         reverse order, so n sweeps apply the polynomial of
                         T^-1 A that damps that interval best (FGMRES
                         iterations on the 256x128x128 sphere grid: 8 -> 7 with
                         3 sweeps on every level, where constant omega needed 5
                         on the coarse levels) */
  double cheb_hi;     /* upper end of the damped interval (default 2: T^-1 A of a
                         diagonally dominant M-matrix has its spectrum in (0, 2]) */
  double cheb_ratio;  /* cheb_hi over the lower end (default 6) */
  int proj_exact;     /* projection of a projection step.  0 (the default): on
                         face weights precomputed with the operator
                         (vfs_projection_faces: the same products, applied with
                         FMAs; within 1e-14 relative of the reference's
                         operation order).  1: the reference's operation order
                         bit for bit (vfs_projection). */
  int mg_grouped;     /* batched solves (vfs_projection_step_batch): 1: the
                         V-cycles of the grids that allow it (full coarsening,
                         not the FP16 operator) run as grouped launches: grids
                         of one precision, level count and size class (cell
                         count within a factor of two) share one chain of
                         launches, operation i of each grid's V-cycle in one
                         launch per kernel with a table of one item per grid,
                         bit for bit the per-grid launches' results.  0 (the
                         default): each grid's own launches, each grid a branch
                         of the tick's graph, which measured faster on GB300
                         (64-grid batch: 877 against 754 solves/s).  Single
                         solves and served requests ignore it. */
  int mg_stage;       /* How the finest level's sweeps on the FP32 face form
                         (levels of at least 2^20 interior cells) stage their
                         operands; both choices give the same results bit for
                         bit.  0 (the default): in registers, four blocks per
                         SM.  1: tensor-memory copies (mx and my even): one
                         block per SM, a producer thread copying 16-row bands
                         of x, the face weights, b and 1/m into a shared-
                         memory ring (cp.async.bulk.tensor, mbarrier
                         completion) while eight warps form residuals, solve
                         columns and write; measured slower on GB300 (the
                         copies alone take as long as the register-staged
                         sweep). */
} vfs_solve_params;
/* The outer FGMRES iterates on the aj-scaled system (aj A) phi = aj b, the
 * form the reference's multigrid path assembles (poisson == -1 scales every
 * row by aj, poisson.c:1560, with the RHS scaled alike).  Its residual r_s =
 * aj (b - A phi) is, cell by cell, the divergence the projection leaves
 * divided by dt st / coeff, so the solve stops when ||r_s|| <= rtol ||aj b||
 * and, when div_tol > 0, the masked max of dt st / coeff * |r_s| (the
 * divergence the projection will leave) is at most div_tol.  A projection
 * step then measures max |div u|.  Where FP64 rounding keeps the masked max
 * above the target (large |phi| on strongly stretched grids: the solve rounds
 * stop once another round no longer halves it), or the rounding of the flux
 * update left it above div_tol, one more projection pass on the corrected
 * fluxes removes the rest (at most two; each solves for the small remaining
 * phi, whose rounding floor is far lower).  The aj-scaled operator drops
 * entries after scaling (|aj v| <= 1e-10, the multigrid path's form,
 * poisson.c:1560, 1607-1616), so it is consistent with the projection even
 * where aj is large. */

typedef struct {
  int iterations;  /* preconditioner applications */
  int converged;
  double relres;   /* true ||aj (b - A phi)|| / ||aj b|| at exit */
  double bnorm;
  double time_ms;  /* device time of the solve */
  int div_limited; /* 1: div_tol was not reached: after a projection step, the
                      measured max |div u| is above div_tol after every
                      projection pass; for a solve alone, the masked residual
                      max stopped falling (the FP64 rounding floor of phi) */
  int mg_half_used; /* 1: the multigrid ran on the FP16 normalised operator
                       (mixed precision, mg_half = 1, and every normalised
                       coefficient of the grid within 6e4; else FP32) */
} vfs_solve_info;

/* Context (device, streams, HBM budget). */
int vfs_create(const vfs_config* cfg, vfs_ctx** out);
void vfs_destroy(vfs_ctx* ctx);
const char* vfs_last_error(const vfs_ctx* ctx);
void vfs_default_params(vfs_solve_params* p);

/* MG_Initial + FormMetrics (init.c:205-905, metrics.c:4-1290): uploads the
 * node coordinates and nvert, builds the coarse levels (every other node,
 * init.c:397-449; MyNvertRestriction, poisson.c:2004-2106) and the metrics
 * of every level on the GPU.  *grid_id receives the handle. */
int vfs_grid_create(vfs_ctx* ctx, const vfs_grid_desc* desc, int* grid_id);
int vfs_grid_destroy(vfs_ctx* ctx, int grid);
/* Device bytes held by a grid (for admission control). */
int vfs_grid_bytes(vfs_ctx* ctx, int grid, unsigned long long* bytes);
/* Bytes a grid with this description would hold (nothing is allocated). */
int vfs_grid_estimate(const vfs_grid_desc* desc, int restart, unsigned long long* bytes);

/* PoissonLHSNew (poisson.c:976-1691): the g tensor and the 19-point
 * coefficients of every level, plus the coarsest-level dense inverse. */
int vfs_poisson_lhs(vfs_ctx* ctx, int grid);

/* Field transfer between host and the resident device state. */
int vfs_set_field(vfs_ctx* ctx, int grid, int field, const double* host);
int vfs_get_field(vfs_ctx* ctx, int grid, int field, double* host);

/* VolumeFlux (poisson.c:2634-2828 / 2898-3240) on the resident Ucont.
 * out[0..3] = IB flux and area before, flux and area after the balance. */
int vfs_volume_flux(vfs_ctx* ctx, int grid, double out[4]);

/* PoissonRHS2_hypre (poisson_hypre.c:342-429) on the resident Ucont, plus
 * the compatibility fix of PoissonRHS2 (poisson.c:1879-1903) when meanfix.
 * *sum_out (nullable) receives the sum of b before the fix. */
int vfs_poisson_rhs(vfs_ctx* ctx, int grid, double dt, double st, double coeff, int meanfix, double* sum_out);

/* PoissonSolver_MG (mhv_poisson.c:2121-2359): FGMRES preconditioned by a
 * geometric V-cycle, then Remove_Nullspace (poisson_hypre.c:207-270) and
 * Convert_Phi2_Phi (poisson.c:97-185) on the resident phi. */
int vfs_poisson_solve(vfs_ctx* ctx, int grid, const vfs_solve_params* p, vfs_solve_info* info);

/* UpdatePressure (poisson.c:2473-2632): p += phi on fluid cells. */
int vfs_update_pressure(vfs_ctx* ctx, int grid);

/* Projection (poisson.c:2122-2470) on the resident Ucont, then Contra2Cart
 * (rhs.c:52-190) into the resident Ucat. */
int vfs_projection(vfs_ctx* ctx, int grid, double dt, double st, double coeff);

/* The same projection on per-face weights formed once by vfs_poisson_lhs:
 * every regime choice of Projection (poisson.c:2221-2363: faces touching
 * nvert skipped; each cross derivative centred, one-sided or absent) depends
 * on the grid only, so it is folded into the weights (dot product times the
 * face Jacobian times 0.25, 0.5 or 0) and two code bits per cross term.  The
 * update is U -= (wN dphi_n + wA dphi_A + wB dphi_B) dt st / coeff with FMAs:
 * about half the FP64 operations of the reference's order, no nvert reads,
 * equal to vfs_projection within 1e-14 relative.  Then Contra2Cart. */
int vfs_projection_faces(vfs_ctx* ctx, int grid, double dt, double st, double coeff);

/* Divergence (main.c:1244-1390): max |div U| * aj over the fluid. */
int vfs_divergence_max(vfs_ctx* ctx, int grid, double* out);

/* Allocation-free variant of the divergence check.  It has no counterpart in
 * the reference: the reference's Divergence (main.c:1244-1390) works on its
 * own PETSc vectors, while this entry point takes caller-owned device arrays
 * and allocates nothing (no cudaMalloc/cudaFree or other allocating call).
 *
 * Who needs it: a caller that must not allocate device memory while a step is
 * in flight, e.g. a host time loop that has handed all of HBM to its own
 * allocator, or one that cannot afford the device-wide synchronisation
 * cudaFree implies while other streams are busy; such a caller has no vfs_ctx
 * and no grid buffers to lend.
 *
 * What it does: max over interior cells of |div U| * aj, 0 where the cell or
 * a face neighbour has nvert (the same kernels as vfs_divergence_max), for
 * the ghosted grid mx x my x mz ([mz][my][mx], i fastest), contravariant
 * fluxes as three component arrays ucont_x/_y/_z, aj and nvert,
 * all device pointers on `device`.  The result is written to the device
 * double *out, ordered on `stream` (a cudaStream_t; NULL = legacy default
 * stream); the call does not synchronise.
 *
 * Scratch: the per-block maxima live in a file-scope static device array of
 * 2432 doubles (19 KB) per device.  Nothing in it has to start at zero (every
 * block writes its entry before the final reduction reads it).  Limits:
 * grids of 2^31 cells or more (ghosts included) are rejected with
 * VFS_ERR_ARG; `device` must be the calling thread's current device.
 * Because the scratch is shared, calls whose kernels may overlap (different
 * streams, or threads, on the same device without ordering between them)
 * race and give undefined results: order them.  The first call on a device
 * looks up the scratch address (cudaGetSymbolAddress, with that device
 * current) and should come before any stream capture; the address is kept
 * for the life of the process, so the device must not be reset
 * (cudaDeviceReset) between calls.  Periodic axes: the flags are accepted
 * but unused; like the reference's Divergence (main.c:1279-1349) the check
 * reads each cell's west, south and back faces at index - 1, so a periodic
 * axis's ghost faces (index 0 = index m - 2) must be filled before the call.
 * err (may be NULL) receives a message of at most err_len - 1 characters. */
int vfs_divergence_max_noalloc(int device, int mx, int my, int mz, int i_periodic, int j_periodic, int k_periodic,
                               const double* ucont_x, const double* ucont_y, const double* ucont_z, const double* aj,
                               const double* nvert, double* out, void* stream, char* err, int err_len);

/* The pressure section of Flow_Solver (solvers.c:871-931): VolumeFlux,
 * PoissonRHS, the solve, UpdatePressure, Projection, Divergence.
 * ucont_inout (nullable): host U* in, corrected U out; when NULL the
 * resident U* (VFS_FIELD_USTAR) is the input and the result stays resident.
 * p_inout (nullable): host pressure in and out.  divmax (nullable). */
int vfs_projection_step(vfs_ctx* ctx, int grid, double* ucont_inout, double* p_inout, double dt, double st,
                        double coeff, const vfs_solve_params* p, vfs_solve_info* info, double* divmax);

/* ---- moving bodies and deforming grids ----
 * New nvert (IB cells moved; the reference rebuilds its LHS then,
 * poisson_hypre.c:628-648) or new node coordinates (moving or deforming
 * grid): the coarse masks and nodes, the metrics of every level, the
 * restriction weights and the inverse metric are rebuilt on the device
 * from the host array ([mz][my][mx] / [mz][my][mx][3]); the grid then needs
 * vfs_poisson_lhs again before its next solve.  Resident U*, p and phi are
 * kept. */
int vfs_grid_update_nvert(vfs_ctx* ctx, int grid, const double* nvert);
int vfs_grid_update_coords(vfs_ctx* ctx, int grid, const double* coor);

/* ---- PETSc binary Vec files ----
 * The reference's field files (vfield/pfield/nvfield/ufield, VecView and
 * VecLoad, main.c:291-330): int32 class id 1211214, int32 length n, then n
 * IEEE doubles, all big-endian.  A DMDA vector is stored in natural ordering,
 * which is this ABI's host layout ([mz][my][mx], Cmpnts as 3 consecutive
 * doubles).  read: out == NULL only returns the file's length in *n_file;
 * otherwise n must equal it.  Host only (no context, no device). */
int vfs_petsc_vec_read(const char* path, double* out, long long n, long long* n_file);
int vfs_petsc_vec_write(const char* path, const double* in, long long n);

/* ---- test and introspection hooks (same arithmetic as the hot path) ---- */
/* metric pack of a level: 43 * N doubles (csi eta zet aj icsi ieta izet iaj
 * jcsi jeta jzet jaj kcsi keta kzet kaj cent; vectors AoS). */
int vfs_get_metrics(vfs_ctx* ctx, int grid, int level, double* out);
/* 19 * N coefficients of a level: which 0 = unscaled FP64 (the outer
 * operator on the finest level), 1 = aj-scaled FP64, 2 = aj-scaled FP32
 * (returned as doubles). */
int vfs_get_coef(vfs_ctx* ctx, int grid, int level, int which, double* out);
/* The FP16 diagonal-normalised multigrid operator of a level (mg_half):
 * coef 19 * N values (slot m != 0: fp16(a_m / D); slot 0: the fp16 row-sum
 * correction), lf N FP32 y-line pivots 1/m (0 on non-fluid rows), rw N FP32
 * restriction weights max(0, 1 - nvert_f) D_f / D_c (level >= 1; zeros on
 * level 0), all returned as doubles; any pointer may be null. */
int vfs_get_mg_half(vfs_ctx* ctx, int grid, int level, double* coef, double* lf, double* rw);
int vfs_get_level_dims(vfs_ctx* ctx, int grid, int level, int dims[3]);
int vfs_get_level_nvert(vfs_ctx* ctx, int grid, int level, double* out);
/* y = A x with the operator `which` (as vfs_get_coef) of a level; which 3 =
 * the aj-scaled FP64 operator applied to x rounded to FP32 (the Krylov
 * product of the mixed-precision solve). */
int vfs_apply_op(vfs_ctx* ctx, int grid, int level, int which, const double* x, double* y);
/* One multigrid preconditioner application z = M^{-1} v on the finest level,
 * issued as the iterations of a lone solve issue it. */
int vfs_apply_precond(vfs_ctx* ctx, int grid, int precision, const vfs_solve_params* p, const double* v, double* z);
/* MyRestriction of level `level` (>= 1) to level-1, MyInterpolation of level-1
 * to `level` (overwrite), in FP64. */
int vfs_mg_restrict(vfs_ctx* ctx, int grid, int level, const double* x, double* y);
int vfs_mg_prolong(vfs_ctx* ctx, int grid, int level, const double* x, double* y);
/* One damped y-line Jacobi sweep on a level (FP64 aj-scaled operator). */
int vfs_mg_smooth(vfs_ctx* ctx, int grid, int level, const double* b, double* x, double omega);
/* Connected fluid regions (cells with nvert < 0.1, joined through shared
 * faces, periodic wrap included) of the finest and the coarsest level, as
 * found by vfs_poisson_lhs.  A grid that bodies cut apart has one constant
 * null vector per region: the step's compatibility fix and the solution's
 * mean removal then act per region, and the coarsest dense solve adds one
 * sigma e_q e_q^T per region (the reference's two-region case:
 * FullyBlocked, poisson.c:1918-1998, and PoissonNullSpaceFunction,
 * poisson.c:819-873). */
int vfs_grid_components(vfs_ctx* ctx, int grid, int* finest, int* coarsest);
/* Damping of the smoothing sweeps the V-cycle launches under p (host only,
 * no device): finest != 0 for the finest level, else the coarser ones;
 * post != 0 for the post-sweeps.  n must equal that side's sweep count.
 * VFS_ERR_ARG for invalid parameters. */
int vfs_sweep_damping(const vfs_solve_params* p, int finest, int post, double* w, int n);
/* Test hook of the tensor-copy sweep (mg_stage = 1): from the next launch on,
 * its producer leaves out the 1/m copies of band `band` of every block (-1,
 * the default: none), so that band's bounded wait (about 0.2 s) runs out;
 * the solve or preconditioner call then fails with VFS_ERR_CUDA ("a bounded
 * wait ran out") and the context stays usable.  Process-wide; returns
 * VFS_OK. */
int vfs_debug_tma_drop(int band);

/* ---- serving: continuous batching of projection steps ----
 * A request is one projection step of one grid (the simulation stream's
 * resident grid: MG hierarchy, pressure and phi stay on the device between
 * its requests).  vfs_submit admits it at once if a slot is free, the grid
 * has no request in flight and the grid's solver memory fits the HBM budget
 * (it is reserved at admission); its inputs and right-hand side go to the
 * device immediately and its iterations interleave with those of every other
 * request in flight, each on its grid's stream.  vfs_poll advances all of
 * them and returns finished ones.  Host buffers must stay valid until the
 * request's result is returned; page-locked buffers (vfs_host_register) keep
 * the copies asynchronous. */
typedef struct {
  int grid;
  const double* ucont_in;   /* host AoS U* [mz][my][mx][3], or NULL: the resident U* */
  double* ucont_out;        /* host AoS corrected fluxes, or NULL (they stay resident) */
  const double* p_in;       /* host pressure, or NULL: the resident pressure */
  double* p_out;            /* host pressure after the update, or NULL */
  double dt, st, coeff;
  vfs_solve_params params;  /* warm_start = 1: start from the grid's resident phi */
} vfs_request;

typedef struct {
  long long ticket;
  int status;               /* VFS_OK or the request's error code */
  vfs_solve_info info;
  double divmax;            /* max |div u| after the projection */
} vfs_result;

/* VFS_ERR_BUSY: no free slot or the grid is busy (retry after a poll);
 * VFS_ERR_NOMEM: the grid's solver memory does not fit the budget now. */
int vfs_submit(vfs_ctx* ctx, const vfs_request* req, long long* ticket);
/* Advances every request in flight; VFS_OK with one finished result in *out,
 * VFS_ERR_BUSY if none has finished yet (wait = 0; wait = 1 blocks until one
 * has), VFS_ERR_STATE if nothing is in flight. */
int vfs_poll(vfs_ctx* ctx, int wait, vfs_result* out);
int vfs_inflight(vfs_ctx* ctx);
/* Device memory the context holds and its budget (0 = none), in bytes. */
int vfs_memory(vfs_ctx* ctx, unsigned long long* used, unsigned long long* budget);

/* ---- batched solves (many uneven grids, one graph launch per iteration) ---- */
/* Runs vfs_projection_step (resident U*, pressure and fluxes stay resident)
 * on n distinct grids.  Every FGMRES iteration of all grids is one CUDA graph
 * launch (one branch per grid, running concurrently; converged grids skip
 * their kernels).  p points to n_params = 1 (shared) or n (per grid) solve
 * parameter sets; infos and divmax (may be NULL) receive n entries. */
int vfs_projection_step_batch(vfs_ctx* ctx, int n, const int* grids, double dt, double st, double coeff,
                              const vfs_solve_params* p, int n_params, vfs_solve_info* infos, double* divmax);

/* Device synchronisation of all work of a context. */
int vfs_sync(vfs_ctx* ctx);

/* ---- measurement ---- */
#define VFS_PROBE_SMOOTH 1   /* full y-line sweeps of the finest multigrid level */
#define VFS_PROBE_APPLY64 2  /* FP64 outer operator apply (w = A z) */
#define VFS_PROBE_ALL 3      /* every instrumented launch of the step (per record: kernel, level) */
/* Record a CUDA event pair around every launch of one kernel (on the stream
 * it runs on) until vfs_probe_end, which returns the launch count, their
 * summed device time and their summed algorithmic bytes (the compulsory HBM
 * reads and writes of each launch).  Iteration graphs are not used while a
 * probe is open, and the host checks convergence after every iteration. */
int vfs_probe_begin(vfs_ctx* ctx, int kernel);
int vfs_probe_end(vfs_ctx* ctx, unsigned long long* launches, double* total_ms, double* alg_bytes);
/* Record i (0-based, < launches) of the last probe: kernel name, multigrid
 * level (finest = levels - 1), device time and algorithmic bytes. */
int vfs_probe_record(vfs_ctx* ctx, int i, char* name, int name_len, int* level, double* ms, double* alg_bytes);
/* CUDA event `slot` (0..4095) recorded on the stream of a grid; elapsed
 * device time between two recorded slots. */
int vfs_mark(vfs_ctx* ctx, int grid, int slot);
int vfs_elapsed(vfs_ctx* ctx, int slot_a, int slot_b, double* ms);
/* Kernels launched by this library since it was loaded (all contexts). */
int vfs_launch_count(unsigned long long* out);
/* Page-lock a host buffer so vfs_projection_step copies it asynchronously. */
int vfs_host_register(void* ptr, unsigned long long bytes);
int vfs_host_unregister(void* ptr);
/* Page-locked host allocation (cudaHostAlloc) for step buffers; on GB300
 * (Grace host) uploads from it run about 10% faster than from registered
 * pageable memory.  VFS_ERR_NOMEM when the allocation fails. */
int vfs_host_alloc(void** ptr, unsigned long long bytes);
int vfs_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif
