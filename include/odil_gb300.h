/*
 * odil_gb300.h -- C ABI of the GB300-native ODIL engine (libodil_gb300.so).
 *
 * Conventions (every entry point):
 *   - plain C types only; device pointers are caller-owned and must point to
 *     memory on the current CUDA device; fields are C-order arrays of the grid
 *     shape (time is the slowest axis);
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream);
 *     calls are asynchronous on that stream and reentrant per stream;
 *   - return 0 (ODIL_OK) or a negative ODIL_ERR_* code; nothing throws;
 *   - no entry point allocates device memory: kernels that need scratch take a
 *     caller workspace sized by the matching *_workspace_bytes() query.
 *     A workspace must be zero-filled once when it is allocated; the kernels
 *     leave it zeroed again after every call.
 *
 * Reference interfaces are cited as file:line of the reference project
 * odil22/odil (paths relative to its code/ directory).
 */
#ifndef ODIL_GB300_H
#define ODIL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ODIL_OK 0
#define ODIL_ERR_SHAPE (-1)     /* sizes out of range or inconsistent */
#define ODIL_ERR_DTYPE (-2)     /* unsupported precision combination */
#define ODIL_ERR_ALIGN (-3)     /* pointer misaligned for vector access */
#define ODIL_ERR_LAUNCH (-4)    /* CUDA launch or runtime failure */
#define ODIL_ERR_TIMEOUT (-5)   /* a bounded device-side wait gave up */
#define ODIL_ERR_NONFINITE (-6) /* NaN/Inf detected in a reduction */
#define ODIL_ERR_WORKSPACE (-7) /* workspace missing or too small */
#define ODIL_ERR_ARG (-8)       /* null pointer or invalid scalar argument */

/* Library version as MAJOR*10000 + MINOR*100 + PATCH.
 * No counterpart in the reference (library metadata). */
int odil_version(void);
/* Static, human-readable text for a status code.
 * No counterpart in the reference (the C ABI reports errors by status). */
const char* odil_status_string(int status);

/* ------------------------------------------------------------------------
 * 1D wave operator on the (t, x) space-time grid.
 *
 * Replaces wave.py:67-122 (operator_fd) evaluated through
 * util_op.py:508-563 (Context.field = periodic roll), with the residual
 *   row 0      f = u - (init_u + dt/2 * init_ut)
 *   row 1      f = ((u - u[i-1])/dt - init_ut)/dt - c^2 u_xx[i-1]
 *   row >= 2   f = (u - 2u[i-1] + u[i-2])/dt^2 - c^2 u_xx[i-1]
 * and u_xx's x-halo replaced by quadratic extrapolation to the Dirichlet
 * values left_u / right_u (util_op.py:1017-1023).  c = 1 is the reference.
 * ---------------------------------------------------------------------- */
typedef struct odil_wave_params {
    int64_t nt, nx;      /* grid cells in t and x */
    double dt, dx;       /* cell sizes */
    double c;            /* wave speed */
    /* Boundary data, device arrays in the kernel's precision (float for
     * *_f32 entry points, double for *_f64).  NULL means zero. */
    const void* init_u;  /* [nx] u(x, t=0) at x cell centres */
    const void* init_ut; /* [nx] u_t(x, t=0) */
    const void* left_u;  /* [nt] u at x = lower, t cell centres */
    const void* right_u; /* [nt] u at x = upper */
} odil_wave_params;

/* Workspace bytes needed by odil_wave_loss_grad_*.
 * Scratch of the loss reduction of util_op.py:627-654; no counterpart (the
 * reference allocates through TF). */
int64_t odil_wave_workspace_bytes(const odil_wave_params* p);

/* f = F(u).  Replaces Problem.eval_operator (util_op.py:968-973) for
 * operator_fd. */
int odil_wave_residual_f32(const odil_wave_params* p, const float* u, float* f,
                           void* stream);
int odil_wave_residual_f64(const odil_wave_params* p, const double* u,
                           double* f, void* stream);

/* Fused adjoint: *loss = mean(f^2), grad = (2/N) J^T f, f = F(u) recomputed
 * in shared-memory tiles and never stored.  Replaces Problem._eval_loss /
 * eval_loss_grad (util_op.py:627-654, 939-966) for operator_fd.  The loss is
 * accumulated in FP64 by a deterministic two-level tree.  If the loss is not
 * finite, *loss holds it and ODIL_OK is still returned (the caller decides). */
int odil_wave_loss_grad_f32(const odil_wave_params* p, const float* u,
                            float* grad, double* loss, void* workspace,
                            int64_t workspace_bytes, void* stream);
int odil_wave_loss_grad_f64(const odil_wave_params* p, const double* u,
                            double* grad, double* loss, void* workspace,
                            int64_t workspace_bytes, void* stream);

/* Allocation-free odil_wave_loss_grad_f32.  No counterpart in the
 * reference: it serves callers that cannot allocate device memory (a host
 * whose memory pool is sealed at start-up, a fixed-budget real-time loop, a
 * plugin given no allocator).  The reduction scratch is a 256 KiB
 * file-scope device array held by every GPU that loads the library, so:
 *   - grids needing more than odil_wave_loss_grad_noalloc_max_blocks()
 *     reduction blocks are rejected with ODIL_ERR_WORKSPACE.  A block is a
 *     tile of the fused kernel (64 x 240 cells for large grids whose rows
 *     are 16-byte aligned, 32 x 120 otherwise), so about 5e8 or 1.2e8
 *     cells fit: 16384 x 16384 (aligned) does, 65536 x 8192 does not;
 *   - all calls share that array: calls that overlap on the GPU race;
 *   - the first call on each device looks up the array's address; make it
 *     before any stream capture.  The address is cached per device (an
 *     atomic, safe for host threads that call at once) and belongs to the
 *     device's primary context: after cudaDeviceReset the entry point must
 *     not be called again in the same process. */
int64_t odil_wave_loss_grad_noalloc_max_blocks(void);
int odil_wave_loss_grad_f32_noalloc(const odil_wave_params* p, const float* u,
                                    float* grad, double* loss, void* stream);

/* out = J v  (matrix-free; replaces the CSR product of util_op.py:877-896). */
int odil_wave_jv_f32(const odil_wave_params* p, const float* v, float* out,
                     void* stream);
int odil_wave_jv_f64(const odil_wave_params* p, const double* v, double* out,
                     void* stream);
/* out = J^T w.
 * The transposed CSR product J^T w that linsolver.py:37-41 forms. */
int odil_wave_jtv_f32(const odil_wave_params* p, const float* w, float* out,
                      void* stream);
int odil_wave_jtv_f64(const odil_wave_params* p, const double* w, double* out,
                      void* stream);
/* The normal-equation matrix J^T J of linsolver.py:35-41, never formed:
 * out = J^T J v in one pass (the fused adjoint with zero boundary data; the
 * workspace, sized by odil_wave_jtj_workspace_bytes and zero-filled once,
 * holds its reduction scratch), and out = diag(J^T J). */
int64_t odil_wave_jtj_workspace_bytes(const odil_wave_params* p);
int odil_wave_jtj_v_f32(const odil_wave_params* p, const float* v, float* out,
                        void* workspace, int64_t workspace_bytes,
                        void* stream);
int odil_wave_jtj_v_f64(const odil_wave_params* p, const double* v,
                        double* out, void* workspace, int64_t workspace_bytes,
                        void* stream);
int odil_wave_jtj_diag_f32(const odil_wave_params* p, float* out, void* stream);
int odil_wave_jtj_diag_f64(const odil_wave_params* p, double* out,
                           void* stream);

/* Direct solve of J x = b by forward substitution along t (J is lower
 * triangular in C order).  Same solution as the normal equations that
 * linsolver.py:35-45 factorizes with SuperLU.  One thread block marches the
 * rows; nx <= 2048. */
int odil_wave_march_f32(const odil_wave_params* p, const float* b, float* x,
                        void* stream);
int odil_wave_march_f64(const odil_wave_params* p, const double* b, double* x,
                        void* stream);

/* One fully parallel FP64 step of a mixed-precision Newton epoch
 * (util.py:242-268 with linsolver.py:28-45, the FP64 residual of the
 * iterative refinement): u_out = u + d (d = FP32 correction from
 * odil_wave_march_f32, or NULL: then u_out is not written and u is used),
 * r = F(u_out) in FP64, rhs = (float)(-r) for the next FP32 solve, and, if
 * rnorm2 != NULL, *rnorm2 = sum(r^2) (FP64, deterministic; needs the
 * workspace).  u_out must not alias u.  `p` carries FP64 boundary data. */
int64_t odil_wave_update_residual_workspace_bytes(const odil_wave_params* p);
int odil_wave_update_residual_mixed(const odil_wave_params* p, const double* u,
                                    const float* d, double* u_out, float* rhs,
                                    double* rnorm2, void* workspace,
                                    int64_t workspace_bytes, void* stream);

/* rhs = (float)(-F(0)): the first right-hand side of a mixed Newton solve
 * from u = 0.  FP64 work only where boundary data enter (rows 0 and 1,
 * columns 0 and nx-1); all other cells are 0.
 * Part of the Newton step of util.py:242-268 (-F at the start state). */
int odil_wave_initial_rhs_mixed(const odil_wave_params* p, float* rhs,
                                void* stream);
/* Number of boundary cells of the grid (rows 0 and 1, then columns 0 and
 * nx-1 of each further row): the length of the table below.
 * No counterpart in the reference (a size query). */
int64_t odil_wave_boundary_cells(const odil_wave_params* p);
/* tbl = (float)(-F(0)) at the boundary cells only, in the order above (rows
 * 0 and 1 in full, then column 0 and column nx-1 of each row from 2): the
 * input of odil_wave_march_tiled_table_f32, which takes the interior as
 * zero.  Same values as odil_wave_initial_rhs_mixed at those cells.
 * Part of the Newton step of util.py:242-268 (-F at the start state). */
int odil_wave_initial_table_mixed(const odil_wave_params* p, float* tbl,
                                  void* stream);
/* rhs = (float)(-F(hi + lo)) for a field held as the unevaluated sum of two
 * FP32 arrays (lo may be NULL): the right-hand side of a mixed Newton epoch
 * whose iterate is kept as FP32 corrections, without an FP64 state.
 * Interior cells are evaluated with exact FP32 products and compensated sums
 * (about 2^-48 of the largest stencil term); boundary cells (rows 0, 1 and
 * columns 0, nx-1) in FP64.  p's boundary arrays are FP64.  Replaces the
 * residual evaluation of util_op.py:859-937 inside the Newton loop. */
int odil_wave_pair_residual_mixed(const odil_wave_params* p, const float* hi,
                                  const float* lo, float* rhs, void* stream);
/* odil_wave_march_f32 with an explicit launch shape: cpt columns per thread
 * (1, 2, 4, 8) and pf right-hand-side rows prefetched into registers (8,
 * 16); the block (nx / cpt threads rounded up to 32) may hold at most 1024,
 * 512 or 256 threads for cpt pf <= 16, <= 32 or more (ODIL_ERR_SHAPE).
 * The direct solve of linsolver.py:35-45, as odil_wave_march_f32. */
int odil_wave_march_shape_f32(const odil_wave_params* p, const float* b,
                              float* x, int32_t cpt, int32_t pf, void* stream);

/* odil_wave_march_* spread over one thread-block cluster: each warp owns
 * 32 cpt - 2 halo columns and marches them with `halo` extra columns on each
 * side for `halo` rows between halo exchanges (the halo columns are
 * recomputed, then refreshed from the neighbours), with pf right-hand-side
 * rows in flight per thread.  Same arithmetic per cell as the single-block
 * march.  exchange 0: cluster barrier, then the halo is reloaded from the
 * stored solution; (cpt, halo, pf) in (4, 32, 16), (4, 48, 16), (8, 96, 16).
 * exchange 1: the neighbours push their edge columns into the warp's shared
 * memory (st.async, mbarrier wait bounded at 1 s; a warp whose wait gives up
 * writes NaN from then on and counts the failure); (cpt, halo, pf) in
 * (2, 16, 16), (4, 8, 8), (4, 16, 16), (4, 24, 8), (4, 32, 16), (8, 32, 16),
 * (8, 64, 16).  FP64: cpt pf <= 64.  warps = tiles per block, 1..4; the
 * cluster (ceil(nx / (32 cpt - 2 halo)) / warps blocks) must hold at most 16
 * blocks and fit on the device; nx >= 2.  ODIL_ERR_SHAPE otherwise.
 * The direct solve of linsolver.py:35-45, as odil_wave_march_f32. */
int odil_wave_march_tiled_f32(const odil_wave_params* p, const float* b,
                              float* x, int32_t cpt, int32_t halo, int32_t pf,
                              int32_t warps, int32_t exchange, void* stream);
int odil_wave_march_tiled_f64(const odil_wave_params* p, const double* b,
                              double* x, int32_t cpt, int32_t halo, int32_t pf,
                              int32_t warps, int32_t exchange, void* stream);
/* odil_wave_march_tiled_f32 of the first correction from u = 0, reading the
 * boundary table of odil_wave_initial_table_mixed instead of a full
 * right-hand side (zero inside): bitwise the result of
 * odil_wave_initial_rhs_mixed followed by odil_wave_march_tiled_f32.
 * Needs nx > cpt (ODIL_ERR_SHAPE otherwise).
 * The direct solve of linsolver.py:35-45 on the first Newton step. */
int odil_wave_march_tiled_table_f32(const odil_wave_params* p,
                                    const float* tbl, float* x, int32_t cpt,
                                    int32_t halo, int32_t pf, int32_t warps,
                                    int32_t exchange, void* stream);
/* Test hook of the bounded halo wait: odil_wave_march_tiled_f32 with
 * exchange 1 whose every wait expects `missing_bytes` (1..65536) more than
 * ever arrive, so each wait gives up after its limit. */
int odil_wave_march_tiled_planted_wait_f32(const odil_wave_params* p,
                                           const float* b, float* x,
                                           int32_t cpt, int32_t halo,
                                           int32_t pf, int32_t warps,
                                           int32_t missing_bytes,
                                           void* stream);
/* Number of halo waits that gave up since the last reset (synchronises the
 * device).
 * No counterpart in the reference (diagnostics of the bounded wait). */
int odil_wave_march_tiled_wait_failures(int64_t* count, int32_t reset);

/* ------------------------------------------------------------------------
 * Batched wave instances of uneven sizes (the reference runs them as
 * separate processes, vary_wave.py:7-43).  Fields of all instances are
 * packed back to back in one array; each instance's first cell `offset` is
 * a multiple of 4.
 * ---------------------------------------------------------------------- */
typedef struct odil_wave_instance {
    int64_t nt, nx;
    double dt, dx, c;
    int64_t offset;    /* first cell in the packed field arrays */
    int64_t offset_x;  /* first entry in packed init_u / init_ut */
    int64_t offset_t;  /* first entry in packed left_u / right_u */
    /* Derived constants, filled on the device by odil_wave_batch_setup. */
    double inv_dt, inv_dx2, c2, dt2, lam2;
    double a, b, half_dt;  /* 1/dt^2, c^2/dx^2, dt/2 */
    float ah, al, ch, cl, bh, bl;  /* A, 2B - 2A, -B as FP32 hi + lo */
} odil_wave_instance;

typedef struct odil_wave_batch {
    int32_t ninst;
    int32_t max_nx;                  /* largest nx of the batch (<= 4096) */
    int64_t total_cells;             /* packed array length */
    odil_wave_instance* inst;        /* device [ninst], sorted by offset */
    const int32_t* order;            /* device [ninst]: march order */
    const void* init_u;              /* device, packed, FP64 */
    const void* init_ut;
    const void* left_u;
    const void* right_u;
    const int32_t* row_inst;         /* device [total_rows]: instance of each
                                        packed time row (rows of instance q
                                        start at inst[q].offset_t) */
    int64_t total_rows;
    const int64_t* bnd_off;          /* device [ninst]: first boundary cell of
                                        each instance in the boundary-cell
                                        sequence (rows 0, 1, then columns 0
                                        and nx-1 of rows 2..) */
    int64_t total_bnd;
} odil_wave_batch;

/* Loss and fused adjoint gradient of every instance in one launch (FP32):
 * loss[i] = mean(f_i^2) over instance i's cells, grad_i = (2/N_i) J_i^T f_i
 * (util_op.py:627-654 per instance), total = sum_i loss[i] (the loss of the
 * batch as one optimisation problem).  The work is split into items
 * (strips of columns by tiles of rows) numbered instance by instance:
 * odil_wave_batch_loss_grad_items(nt, nx) gives an instance's item count;
 * tile_start [ninst + 1]: the first item of each instance (tile_start[ninst]
 * = ntiles, the total); tile_inst [ntiles]: the instance of each item;
 * init_u .. right_u: the packed boundary arrays in FP32; partials: ntiles
 * doubles of scratch; total may be null.  Requires odil_wave_batch_setup.
 * The batched form of the per-run loss of vary_wave.py:37-43. */
int64_t odil_wave_batch_loss_grad_items(int64_t nt, int64_t nx);
int odil_wave_batch_loss_grad_f32(const odil_wave_batch* b,
                                  const int64_t* tile_start,
                                  const int32_t* tile_inst, int64_t ntiles,
                                  const float* init_u, const float* init_ut,
                                  const float* left_u, const float* right_u,
                                  const float* u, float* grad,
                                  double* partials, double* loss,
                                  double* total, void* stream);

/* Fills the derived constants of a device descriptor array.
 * Set-up of the batched solver that replaces the per-instance runs of
 * vary_wave.py:37-43; no direct counterpart. */
int odil_wave_batch_setup(odil_wave_instance* inst, int32_t ninst,
                          void* stream);
int64_t odil_wave_batch_workspace_bytes(const odil_wave_batch* b);
/* FP64 step of a mixed Newton epoch for every instance: as
 * odil_wave_update_residual_mixed on the packed arrays.
 * util.py:242-268 per instance (the batched form of vary_wave.py:37-43). */
int odil_wave_batch_update_residual_mixed(const odil_wave_batch* b,
                                          const double* u, const float* d,
                                          double* u_out, float* rhs,
                                          void* stream);
/* Batched odil_wave_initial_rhs_mixed / odil_wave_pair_residual_mixed on
 * the packed arrays (one block per row task, FP64 only on boundary cells).
 * util.py:242-268 per instance (the batched form of vary_wave.py:37-43). */
int odil_wave_batch_initial_rhs_mixed(const odil_wave_batch* b, float* rhs,
                                      void* stream);
int odil_wave_batch_pair_residual_mixed(const odil_wave_batch* b,
                                        const float* hi, const float* lo,
                                        float* rhs, void* stream);
/* FP32 forward substitution of every instance in one persistent launch:
 * blocks_per_sm x #SM blocks of `threads` threads take instances from an
 * atomic work queue in `order`; threads * cpt >= max_nx; (cpt, pf) in
 * {1, 2, 4} x {8, 16} (pf = prefetched right-hand-side rows).
 * linsolver.py:35-45 per instance (the batched form of vary_wave.py:37-43). */
int odil_wave_batch_march_f32(const odil_wave_batch* b, const float* rhs,
                              float* x, int32_t threads, int32_t cpt,
                              int32_t pf, int32_t blocks_per_sm,
                              void* workspace, int64_t workspace_bytes,
                              void* stream);
/* The whole mixed Newton from u = 0 of every instance in ONE persistent
 * launch: each block takes the next instance (largest first, `order`) from
 * an atomic work queue and runs its epochs as marches whose right-hand sides
 * are formed inside the march from the previous iterate (float pairs inside,
 * FP64 on the boundary cells, computed by the block into a table in the
 * instance's rhs region): hi = J^-1 float(-F(0)), then epochs - 1 times
 * x = J^-1 float(-F(hi + lo)) with lo = x (first) or lo += x, and u = hi + lo
 * in FP64 written by the last march.  Results are bitwise those of
 * odil_wave_batch_initial_rhs_mixed / _march_f32 / _pair_residual_mixed /
 * odil_pair_to_f64 run in that order.  rhs (the boundary tables), hi (and lo
 * for epochs >= 2): packed FP32 scratch; u: the packed FP64 solution.
 * Launch shape as odil_wave_batch_march_f32, with (cpt, pf) in {(1, 8),
 * (1, 16), (2, 8), (4, 8)} and threads <= 1024 (cpt 1) or 512.
 * workspace: 256 bytes, zeroed before the first call (the last block to
 * finish leaves it zeroed again); not shared with odil_wave_batch_march_f32.
 * util.py:242-268 per instance (the batched form of vary_wave.py:37-43). */
int odil_wave_batch_solve_mixed(const odil_wave_batch* b, int32_t epochs,
                                float* rhs, float* hi, float* lo,
                                double* u, int32_t threads, int32_t cpt,
                                int32_t pf, int32_t blocks_per_sm,
                                void* workspace, int64_t workspace_bytes,
                                void* stream);

/* ------------------------------------------------------------------------
 * 2D linear advection on the (t, x, y) space-time grid, periodic in x, y.
 *
 * Replaces advection_2d.py:103-223 (operator, direct problem, --periodic 1,
 * first-order upwind on the frozen velocity) for a constant velocity:
 *   f = (p - ptm)/dt + ax p_x + ay p_y, ptm = p[i-1], row 0: ptm = p_init,
 *   p_x = (p - p[x-1])/dx if ax > 0 else (p[x+1] - p)/dx (same in y).
 * ---------------------------------------------------------------------- */
typedef struct odil_advect_params {
    int64_t nt, nx, ny;  /* grid cells; nt, nx <= 65535 */
    double dt, dx, dy;
    double ax, ay;       /* constant velocity */
    const void* p_init;  /* [nx*ny] previous value of row 0 (the reference's
                            exact_pp[0]); kernel precision; NULL = 0 */
} odil_advect_params;

int64_t odil_advect_workspace_bytes(const odil_advect_params* p);
int odil_advect_residual_f32(const odil_advect_params* p, const float* u,
                             float* f, void* stream);
int odil_advect_residual_f64(const odil_advect_params* p, const double* u,
                             double* f, void* stream);
int odil_advect_jv_f32(const odil_advect_params* p, const float* v,
                       float* out, void* stream);
int odil_advect_jv_f64(const odil_advect_params* p, const double* v,
                       double* out, void* stream);
int odil_advect_jtv_f32(const odil_advect_params* p, const float* w,
                        float* out, void* stream);
int odil_advect_jtv_f64(const odil_advect_params* p, const double* w,
                        double* out, void* stream);
/* Fused loss + adjoint (util_op.py:627-654): *loss = mean(f^2),
 * grad = (2/N) J^T f. */
int odil_advect_loss_grad_f32(const odil_advect_params* p, const float* u,
                              float* grad, double* loss, void* workspace,
                              int64_t workspace_bytes, void* stream);
int odil_advect_loss_grad_f64(const odil_advect_params* p, const double* u,
                              double* grad, double* loss, void* workspace,
                              int64_t workspace_bytes, void* stream);
/* FP64 step of the mixed-precision Newton loop, as
 * odil_wave_update_residual_mixed.
 * The Newton loop of advection_2d.py:527-604 (FP64 residual and update). */
int odil_advect_update_residual_mixed(const odil_advect_params* p,
                                      const double* u, const float* d,
                                      double* u_out, float* rhs,
                                      double* rnorm2, void* workspace,
                                      int64_t workspace_bytes, void* stream);
/* Matrix-free FP32 multigrid on the same operator (the V-cycle of
 * multigrid.py:567-602 with rediscretised coarse operators; coarse levels
 * pass their own params with doubled steps).  Damped Jacobi
 * (multigrid.py:543-552): x_out = x + omega (b - J x)/diag(J); x = NULL means
 * a zero iterate.  r_out (optional, needs x) receives b - J x. */
int odil_advect_mg_jacobi(const odil_advect_params* p, const float* x,
                          const float* b, float* x_out, float omega,
                          float* r_out, void* stream);
/* Full-weighting restriction (nt, nx, ny) -> halves: weights
 * (1, 3, 3, 1)/8 per axis, x and y periodic, t clamped.
 * Restriction of multigrid.py:496-534, rediscretised V-cycle (the reference
 * uses pyamg, linsolver.py:81-89). */
int odil_advect_mg_restrict(int64_t nt, int64_t nx, int64_t ny,
                            const float* r, float* rc, void* stream);
/* x += trilinear prolongation of the half-size correction e.
 * Prolongation of multigrid.py:471-494 (the reference uses pyamg,
 * linsolver.py:81-89). */
int odil_advect_mg_prolong_add(int64_t nt, int64_t nx, int64_t ny,
                               const float* e, float* x, void* stream);
/* Dense FP64 matrix of the operator (nt*nx*ny <= 1024), for the coarsest
 * level's direct solve.
 * Coarsest-level direct solve (multigrid.py:322-323). */
int odil_advect_dense(const odil_advect_params* p, double* A, void* stream);
/* x = Ainv b with a dense FP64 n x n matrix (n <= 1024): the coarsest-level
 * direct solve (multigrid.py:307-310) by the precomputed inverse. */
int odil_dense_apply_f64(int64_t n, const double* Ainv, const float* b,
                         float* x, void* stream);

/* ------------------------------------------------------------------------
 * Steady Navier-Stokes, lid-driven cavity on an n x n grid of [0, 1]^2.
 *
 * Replaces ns_steady.py:142-433 (operator) with its defaults: no-slip walls
 * and lid u = 1 at y = 1 by quadratic extrapolation (bc 0), deferred-
 * correction upwind momentum, central pressure gradient, Rhie-Chow
 * continuity; mu = 1/Re.  Residual terms, in order: fu, fv, fp, then
 * [imposed u, v] (mask != NULL), [kreg u_xx, u_yy, v_xx, v_yy] (kreg != 0),
 * [pin_weight * p at cell `pin`] (pin >= 0, the benchmark's pressure pin).
 * ---------------------------------------------------------------------- */
typedef struct odil_ns_params {
    int64_t n;
    double re;
    double kreg;
    const void* mask;   /* [n*n] imposed-point mask (kernel precision) or NULL */
    const void* u_imp;  /* [n*n] imposed values */
    const void* v_imp;
    double imp_coeff;   /* alpha * n^2 / n_imp (ns_steady.py:400) */
    int64_t pin;        /* flat index of the pinned pressure cell, -1: none */
    double pin_weight;
} odil_ns_params;

/* Number of residual terms for these parameters (or a negative status).
 * The term count of ns_steady.py:388-411. */
int odil_ns_num_equations(const odil_ns_params* q);
/* f[e*n*n + cell] = residual term e at (u, v, p) (frozen = live = state).
 * The residual terms of ns_steady.py:142-433 (util_op.py:968-973). */
int odil_ns_residual_f32(const odil_ns_params* q, const float* u,
                         const float* v, const float* p, float* f,
                         void* stream);
int odil_ns_residual_f64(const odil_ns_params* q, const double* u,
                         const double* v, const double* p, double* f,
                         void* stream);
/* Jacobian in stencil form at the state (util_op.py:585-614):
 * coef[(e*15 + s)*n*n + cell] = d f_e / d (live slot s), s = field*5 + k,
 * field in (u, v, p), k in (c, x-1, x+1, y-1, y+1). */
int odil_ns_jacobian_f32(const odil_ns_params* q, const float* u,
                         const float* v, const float* p, float* coef,
                         void* stream);
int odil_ns_jacobian_f64(const odil_ns_params* q, const double* u,
                         const double* v, const double* p, double* coef,
                         void* stream);

/* Direct solve of the cavity Newton system (3 equations, forward problem:
 * no imposed points, no penalty) with the continuity row of cell `pin`
 * (= i n + j) replaced by p[pin] = value, which makes the square Jacobian
 * nonsingular.  Replaces the SuperLU solve of linsolver.py:28-45 for this
 * family.  coef: the [3][15][n][n] FP64 output of odil_ns_jacobian_f64.
 * The system is block tridiagonal over the first grid axis (blocks of 3n
 * unknowns); factor computes its FP32 block LU (cuSOLVER dense LU per
 * block) into the workspace, solve applies it to an FP32 right-hand side
 * (field-major [3][n][n]) for FP64 iterative refinement by the caller.
 * Workspace: about 8 (3n)^2 n bytes (9.7 GB at n = 512).  check returns the
 * number of blocks with a singular pivot (synchronises the stream). */
int64_t odil_ns_direct_workspace_bytes(int64_t n);
int odil_ns_direct_factor(int64_t n, const double* coef, int64_t pin,
                          void* workspace, int64_t workspace_bytes,
                          void* stream);
int odil_ns_direct_check(int64_t n, const void* workspace, void* stream);
int odil_ns_direct_solve(int64_t n, const double* coef, int64_t pin,
                         void* workspace, int64_t workspace_bytes,
                         const float* b, float* x, void* stream);
/* Explicit inverse of a small dense FP64 matrix (n <= 4096) by cuSOLVER LU
 * with partial pivoting.  Ainv comes out in the layout A goes in (row- or
 * column-major): the inverse of the transpose is the transpose of the
 * inverse.  ODIL_ERR_NONFINITE for an exactly singular matrix; synchronises
 * the stream.
 * Coarsest-level direct solve of multigrid.py:322-323 (spsolve there). */
int64_t odil_dense_inverse_workspace_bytes(int64_t n);
int odil_dense_inverse_f64(int64_t n, const double* A, double* Ainv,
                           void* workspace, int64_t workspace_bytes,
                           void* stream);

/* The transposed solve J'^T x = b with the same factors (the preconditioner
 * (J'^T J')^-1 of the inverse problem's normal equations needs both).
 * Part of the normal-equation solve of linsolver.py:35-45 for the cavity. */
int odil_ns_direct_solve_t(int64_t n, const double* coef, int64_t pin,
                           void* workspace, int64_t workspace_bytes,
                           const float* b, float* x, void* stream);

/* ------------------------------------------------------------------------
 * Cavity multigrid on the normal equations.  The reference solves a Newton
 * (or Gauss-Newton) step J^T J d = -J^T f with V-cycles of its multigrid on
 * J^T J (util.py:509-604 with multigrid.py:429-469, 543-602; the normal
 * equations of linsolver.py:35-45).  Here the levels are cell-centred (n,
 * n/2, ... while even; the reference's node-based transfer needs odd
 * sizes): bilinear prolongation P (3/4, 1/4 per axis, the outer weight moved
 * to the wall cell at a wall), R = P^T / 4, Galerkin R A P.
 *   vectors: [3][n][n] (u, v, p); coef: the [neq][15][n][n] coefficients of
 *   odil_ns_jacobian_*; 25-point operators: [9][25][n][n], block 3 f + g,
 *   point (dx + 2) * 5 + (dy + 2); dinv: [9][n][n] inverses of the 3 x 3
 *   per-cell diagonal blocks.
 * ---------------------------------------------------------------------- */
/* w = J x (the util_op.py:877-896 product, from the stencil coefficients) */
int odil_nsmg_jx_f32(int64_t n, int32_t neq, const float* coef, const float* x,
                     float* w, void* stream);
int odil_nsmg_jx_f64(int64_t n, int32_t neq, const double* coef,
                     const double* x, double* w, void* stream);
/* y = J^T w (linsolver.py:37-41); mode 0: out = y, 1: out = b - y,
 * 2: out = x + omega dinv (b - y) (damped block Jacobi, multigrid.py:
 * 283-299 with the per-cell blocks of multigrid.py:288-295). */
int odil_nsmg_jtw_f32(int64_t n, int32_t neq, const float* coef,
                      const float* w, const float* b, const float* x,
                      const float* dinv, float* out, float omega, int32_t mode,
                      void* stream);
int odil_nsmg_jtw_f64(int64_t n, int32_t neq, const double* coef,
                      const double* w, double* out, void* stream);
/* A = J^T J as 25-point stencils and its block-diagonal inverses (the
 * matrix linsolver.py:35-41 assembles, in stencil form). */
int odil_nsmg_fine_ata(int64_t n, int32_t neq, const float* coef, float* A,
                       float* dinv, void* stream);
/* Ac = R A P on the n/2 grid and its block-diagonal inverses
 * (multigrid.py:125-131, 390-427). */
int odil_nsmg_galerkin(int64_t n, const float* A, float* Ac, float* dinv_c,
                       void* stream);
/* 25-point level operator; mode 0: out = A x, 1: out = b - A x,
 * 2: out = x + omega dinv (b - A x) (multigrid.py:283-299). */
int odil_nsmg_smooth(int64_t n, const float* A, const float* dinv,
                     const float* x, const float* b, float* out, float omega,
                     int32_t mode, void* stream);
/* out = omega dinv b: the first Jacobi sweep from zero. */
int odil_nsmg_jacobi0(int64_t n, const float* dinv, const float* b,
                      float* out, float omega, void* stream);
/* rc = R r on the n/2 grid; x += P e from the n/2 grid (multigrid.py:
 * 590-598, the transfers of a V-cycle). */
int odil_nsmg_restrict(int64_t n, const float* r, float* rc, void* stream);
int odil_nsmg_prolong_add(int64_t n, const float* e, float* x, void* stream);
/* Coarsest level (3 n^2 <= 1024 unknowns): the dense FP64 inverse of the
 * 25-point operator (Gauss-Jordan, one block; a pivot at or below 1e-13 of
 * the largest diagonal entry drops that direction), and x = minv b.
 * Replaces multigrid.py:307-310 (spsolve on the coarsest matrix). */
int odil_nsmg_coarse_inverse(int64_t n, const float* A, double* minv,
                             void* stream);
int odil_nsmg_coarse_apply(int64_t n, const double* minv, const float* b,
                           float* x, void* stream);
/* Preconditioned conjugate gradients with the step scalars on the device
 * (sc = [<r, z>, alpha, beta], FP64).  phase 0: alpha = sc[0] / dots[0]
 * (dots[0] = <p, A p>); phase 1: beta = dots[0] / sc[0], sc[0] = dots[0]
 * (dots[0] = <r, z>); phase 2: sc[0] = dots[0], beta = 0 (first step).
 * update_xr: x += alpha p, r -= alpha q; update_p: p = z + beta p.
 * No counterpart in the reference (its CG is scipy's, on the host). */
int odil_pcg_scalars(const double* dots, double* sc, int32_t phase,
                     void* stream);
int odil_pcg_update_xr(int64_t n, float* x, float* r, const float* p,
                       const float* q, const double* sc, void* stream);
int odil_pcg_update_p(int64_t n, float* p, const float* z, const double* sc,
                      void* stream);

/* ------------------------------------------------------------------------
 * Operators in stencil form (the reference's SparseOperator,
 * multigrid.py:877-1214): shifts s with one coefficient field C_s each on the
 * output grid,  (A u)[c] = sum_s C_s[c] u[stride*c + s], zero outside the
 * grid on non-periodic axes and wrapped on periodic ones.
 * ---------------------------------------------------------------------- */
#define ODIL_STENCIL_MAXS 128

typedef struct odil_stencil {
    int32_t dim;                         /* 1..3 */
    int32_t stride;                      /* 1, or 2 for restriction-type ops */
    int32_t periodic[3];                 /* per axis: 1 = periodic */
    int64_t nw[3];                       /* input (fine) grid */
    int32_t nshift;                      /* <= ODIL_STENCIL_MAXS */
    int32_t shifts[ODIL_STENCIL_MAXS][3];
    void* coef;                          /* device [nshift][output cells],
                                            output grid nwh = (nw-1)/stride+1
                                            (nw/2 on periodic stride-2 axes) */
} odil_stencil;

/* out = beta out + alpha A u  (multigrid.py:958-969, mul_field) */
int odil_stencil_apply_f32(const odil_stencil* A, const float* u, float* out,
                           double alpha, double beta, void* stream);
int odil_stencil_apply_f64(const odil_stencil* A, const double* u,
                           double* out, double alpha, double beta,
                           void* stream);
/* out = beta out + alpha A^T uh  (multigrid.py:1006-1027) */
int odil_stencil_apply_t_f32(const odil_stencil* A, const float* uh,
                             float* out, double alpha, double beta,
                             void* stream);
int odil_stencil_apply_t_f64(const odil_stencil* A, const double* uh,
                             double* out, double alpha, double beta,
                             void* stream);
/* Small device scratch for the two set-up products below.
 * Scratch of the SparseOperator products of multigrid.py:1035-1071, 125-131;
 * no counterpart. */
int64_t odil_stencil_pair_workspace_bytes(void);
/* C = A^T B as a stencil (multigrid.py:1035-1071); C->shifts must list every
 * difference b - a of the shifts of A and B; C->coef is written.  Set-up
 * call: synchronizes the stream. */
int odil_stencil_mul_transpose_op_f32(const odil_stencil* A,
                                      const odil_stencil* B, odil_stencil* C,
                                      void* workspace, int64_t workspace_bytes,
                                      void* stream);
int odil_stencil_mul_transpose_op_f64(const odil_stencil* A,
                                      const odil_stencil* B, odil_stencil* C,
                                      void* workspace, int64_t workspace_bytes,
                                      void* stream);
/* Ac = R A T with T = TT^T, in stencil form: the Galerkin coarse operator of
 * Multigrid.update_A (multigrid.py:125-131).  Ac->shifts list the coarse
 * shifts to produce (|shift| <= 4).  Set-up call: synchronizes the stream. */
int odil_stencil_galerkin_f32(const odil_stencil* R, const odil_stencil* A,
                              const odil_stencil* TT, odil_stencil* Ac,
                              void* workspace, int64_t workspace_bytes,
                              void* stream);
int odil_stencil_galerkin_f64(const odil_stencil* R, const odil_stencil* A,
                              const odil_stencil* TT, odil_stencil* Ac,
                              void* workspace, int64_t workspace_bytes,
                              void* stream);
/* One block row of a coupled system (nterm <= 4 terms A_ij u_j):
 *   r = f - sum_j A_ij u_j  (r_out, optional; f may be NULL = 0),
 *   u_out = u_i + omega r / diag   (optional; damped Jacobi of
 *   multigrid.py:543-552). */
int odil_stencil_block_row_f32(int nterm, const odil_stencil* const* ops,
                               const void* const* us, const float* f,
                               const float* u_i, const float* diag,
                               float* u_out, float* r_out, double omega,
                               void* stream);
int odil_stencil_block_row_f64(int nterm, const odil_stencil* const* ops,
                               const void* const* us, const double* f,
                               const double* u_i, const double* diag,
                               double* u_out, double* r_out, double omega,
                               void* stream);

/* ------------------------------------------------------------------------
 * Optimizer vector kernels (n elements, contiguous).
 * ---------------------------------------------------------------------- */

/* Fused Adam step, the update of optimizer.py:301-314 (AdamNativeOptimizer,
 * the Keras Adam equations):
 *   m += (g - m)(1 - beta1);  v += (g^2 - v)(1 - beta2);
 *   x -= alpha m / (sqrt(v) + epsilon),
 * alpha = lr sqrt(1 - beta2^t) / (1 - beta1^t) computed by the caller. */
int odil_adam_step_f32(float* x, const float* g, float* m, float* v, int64_t n,
                       double alpha, double beta1, double beta2,
                       double epsilon, void* stream);
int odil_adam_step_f64(double* x, const double* g, double* m, double* v,
                       int64_t n, double alpha, double beta1, double beta2,
                       double epsilon, void* stream);

/* z = a x + b y (z may alias x or y); the GD update of optimizer.py:260 and
 * the line-search trial points of the L-BFGS driver. */
int odil_axpby_f32(float* z, const float* x, const float* y, int64_t n,
                   double a, double b, void* stream);
int odil_axpby_f64(double* z, const double* x, const double* y, int64_t n,
                   double a, double b, void* stream);

/* out = u + (double)d (n elements): the FP64 update after the last FP32
 * correction of a mixed-precision Newton solve.
 * The update packed += d of util.py:242-268. */
int odil_add_f32_to_f64(const double* u, const float* d, double* out,
                        int64_t n, void* stream);

/* out = (double)hi + (double)lo (n elements; lo may be NULL): the FP64
 * iterate of a mixed Newton solve kept as FP32 corrections.
 * The update packed += d of util.py:242-268, for the float-pair iterate. */
int odil_pair_to_f64(const float* hi, const float* lo, double* out, int64_t n,
                     void* stream);

/* BiCGStab with device-side scalars (the advection inner solve).  sc is an
 * FP64 [4] array: rho, alpha, omega, beta (start: 1, 1, 1, 0).  scalars:
 * phase 0: rho' = dots[0] = <r^, r>, beta = (rho'/rho)(alpha/omega),
 * rho = rho'; phase 1: alpha = rho / dots[0] (= <r^, v>); phase 2: omega =
 * dots[1] / dots[0] (= <t, s> / <t, t>).  Updates (n % 4 == 0, 16-byte
 * aligned FP32 vectors): p = r + beta (p - omega v); s = r - alpha v;
 * x += alpha ph (+ omega sh), r = s - omega t when with_s.
 * The inner Krylov solve of linsolver.py:75-107 (bicgstab /
 * multigrid-preconditioned). */
int odil_bicgstab_scalars(const double* dots, double* sc, int32_t phase,
                          void* stream);
int odil_bicgstab_update_p(float* p, const float* r, const float* v,
                           const double* sc, int64_t n, void* stream);
int odil_bicgstab_update_s(float* s, const float* r, const float* v,
                           const double* sc, int64_t n, void* stream);
int odil_bicgstab_update_xr(float* x, float* r, const float* ph,
                            const float* sh, const float* s, const float* t,
                            const double* sc, int64_t n, int32_t with_s,
                            void* stream);

/* Multi-dot: out[i*r + j] = sum_e M[i*ld + e] * q[j][e] for i < k, j < r
 * (r <= 4), in one pass over M.  Each thread sums its share of a chunk in
 * the input type (about n * ceil(k/4) / (1824 * 256) products, at least 16), the
 * rest is added in FP64; deterministic order.  The workspace size serves
 * every call with at most k rows and r vectors.
 * This and odil_lincomb_* are the two streaming passes of the compact L-BFGS
 * direction that replaces scipy's fmin_l_bfgs_b (optimizer.py:61-99):
 * [S; Y] . g (plus the new correction pair's products), then
 * d = c0 g + sum_i coef[i] [S; Y]_i.  With more than 8 results a second
 * launch adds the chunk partials, one warp per result. */
int64_t odil_multidot_workspace_bytes(int64_t n, int k, int r);
int odil_multidot_f32(const float* M, int64_t ld, int k, const void* const* q,
                      int r, int64_t n, double* out, void* workspace,
                      int64_t workspace_bytes, void* stream);
int odil_multidot_f64(const double* M, int64_t ld, int k,
                      const void* const* q, int r, int64_t n, double* out,
                      void* workspace, int64_t workspace_bytes, void* stream);

/* out = coef[k] * x + sum_{i<k} coef[i] * M[i*ld ...]; coef is a device array
 * of k+1 doubles; k <= 256.
 * The direction update of the L-BFGS two-loop in optimizer.py:61-99 (scipy
 * there). */
int odil_lincomb_f32(float* out, const float* x, const float* M, int64_t ld,
                     int k, const double* coef, int64_t n, void* stream);
int odil_lincomb_f64(double* out, const double* x, const double* M,
                     int64_t ld, int k, const double* coef, int64_t n,
                     void* stream);
/* odil_lincomb_* that also writes dot[0] = <out, x> (FP64, deterministic):
 * the L-BFGS direction d and phi'(0) = g . d in one pass.  workspace: at
 * least odil_lincomb_dot_workspace_bytes(n) bytes, zeroed before first use
 * (the kernel leaves its counter at zero). */
int64_t odil_lincomb_dot_workspace_bytes(int64_t n);
int odil_lincomb_dot_f32(float* out, const float* x, const float* M,
                         int64_t ld, int k, const double* coef, int64_t n,
                         double* dot, void* workspace, int64_t workspace_bytes,
                         void* stream);
int odil_lincomb_dot_f64(double* out, const double* x, const double* M,
                         int64_t ld, int k, const double* coef, int64_t n,
                         double* dot, void* workspace, int64_t workspace_bytes,
                         void* stream);

/* L-BFGS with the compact-form algebra on the device (replaces the host
 * side of optimizer.py:61-99, scipy's fmin_l_bfgs_b two-loop and line-search
 * driver; the state layout is documented in csrc/lbfgs.cu):
 *   coef: coef[0 .. gidx] of d = -H_k g = sum_{row < gidx} coef[row] H[row]
 *         + coef[gidx] g from the held pairs (compact representation);
 *   trial: xt = x + a d, a = 1 (or min(1, 1/|g|) with no pair held),
 *          phi'(0) = dots[0] recorded;
 *   accept: the Wolfe / approximate-Wolfe test of the trial -> sc[6];
 *   pair: s = a d, y = g_trial - g into sy[0:n], sy[n:2n] (accepted only);
 *   update: ring, S^T Y, Y^T Y, gamma and the dots with the new gradient
 *           from P ([rows][3] dots of H's rows with (g_trial, s, y)) and
 *           Q ([[s.y, s.g_trial], [y.y, y.g_trial]]);
 *   commit: H rows of the updated slot <- (s, y), and g <- g_trial when g
 *           is given (accepted steps only; every kernel after the Wolfe test
 *           is guarded by the status, so an iteration can be enqueued, or
 *           captured in a CUDA graph, before the host reads it). */
int odil_lbfgs_coef(int32_t m, int32_t gidx, const int* ring, const double* SY,
                    const double* YY, const double* dg, const double* sc,
                    double* coef, void* stream);
int odil_lbfgs_trial_f32(int64_t n, float* xt, const float* x, const float* d,
                         const double* dots, const int* ring, double* sc,
                         void* stream);
int odil_lbfgs_trial_f64(int64_t n, double* xt, const double* x,
                         const double* d, const double* dots, const int* ring,
                         double* sc, void* stream);
int odil_lbfgs_accept(const double* ft, const double* dpa, double* sc,
                      void* stream);
int odil_lbfgs_pair_f32(int64_t n, float* sy, const float* d, const float* gt,
                        const float* g, const double* sc, void* stream);
int odil_lbfgs_pair_f64(int64_t n, double* sy, const double* d,
                        const double* gt, const double* g, const double* sc,
                        void* stream);
/* pair_dots: pair, its dots and the Wolfe test in one pass: s = a d,
 * y = g_trial - g into sy (always), Q as for update, and (mode 0) the test
 * of accept on f(trial) = ft[0] with phi'(a) = g_trial . d computed here, or
 * (mode 1) no test: the host chose the step (sc[3], sc[4], sc[6] = 0).
 * workspace: at least odil_lbfgs_pair_dots_workspace_bytes(n) bytes, zeroed
 * before first use. */
int64_t odil_lbfgs_pair_dots_workspace_bytes(int64_t n);
int odil_lbfgs_pair_dots_f32(int64_t n, float* sy, const float* d,
                             const float* gt, const float* g, const double* ft,
                             int32_t mode, double* sc, double* Q,
                             void* workspace, int64_t workspace_bytes,
                             void* stream);
int odil_lbfgs_pair_dots_f64(int64_t n, double* sy, const double* d,
                             const double* gt, const double* g,
                             const double* ft, int32_t mode, double* sc,
                             double* Q, void* workspace,
                             int64_t workspace_bytes, void* stream);
int odil_lbfgs_update(int* ring, double* SY, double* YY, double* dg,
                      double* sc, const double* P, int32_t rows,
                      const double* Q, void* stream);
int odil_lbfgs_commit_f32(int64_t n, float* H, int64_t ld, const float* sy,
                          float* g, const float* gt, const int* ring,
                          const double* sc, void* stream);
int odil_lbfgs_commit_f64(int64_t n, double* H, int64_t ld, const double* sy,
                          double* g, const double* gt, const int* ring,
                          const double* sc, void* stream);

/* ------------------------------------------------------------------------
 * Multigrid decomposition of a field: the field is the sum over levels l of
 * the level-l weights refined l times.
 *
 * Replaces MultigridDecomp.interp_node_field / interp_cell_field
 * (multigrid.py:1220-1362, one level per call) as composed by
 * weights_to_field (multigrid.py:1409-1426); the adjoint replaces the
 * reverse-mode differentiation TensorFlow applies through them.
 * `n` is a host array of `dim` (1..3) coarse sizes.  cell = 0 refines nodes,
 * n -> 2n - 1 per axis (multilinear); cell = 1 refines cells, n -> 2n
 * (weights 3/4, 1/4 over a halo of linearly extrapolated cells; n >= 2).
 * ---------------------------------------------------------------------- */
/* out = alpha * refine(in) + beta * add, on the fine grid; add may be NULL;
 * out must not overlap in or add. */
int odil_mgdecomp_refine_f32(int32_t dim, const int64_t* n, int32_t cell,
                             const float* in, float* out, double alpha,
                             const float* add, double beta, void* stream);
int odil_mgdecomp_refine_f64(int32_t dim, const int64_t* n, int32_t cell,
                             const double* in, double* out, double alpha,
                             const double* add, double beta, void* stream);
/* Adjoint: with a = refine^T g (coarse grid), gc = a and wc = alpha_c * a,
 * and wf = beta_f * g on the fine grid; each of gc, wc, wf may be NULL (not
 * all three); none may overlap g. */
int odil_mgdecomp_refine_t_f32(int32_t dim, const int64_t* n, int32_t cell,
                               const float* g, float* gc, float* wc,
                               double alpha_c, float* wf, double beta_f,
                               void* stream);
int odil_mgdecomp_refine_t_f64(int32_t dim, const int64_t* n, int32_t cell,
                               const double* g, double* gc, double* wc,
                               double alpha_c, double* wf, double beta_f,
                               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ODIL_GB300_H */
