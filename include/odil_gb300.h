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

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int odil_version(void);
/* Static, human-readable text for a status code. */
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

/* Workspace bytes needed by odil_wave_loss_grad_*. */
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

/* out = J v  (matrix-free; replaces the CSR product of util_op.py:877-896). */
int odil_wave_jv_f32(const odil_wave_params* p, const float* v, float* out,
                     void* stream);
int odil_wave_jv_f64(const odil_wave_params* p, const double* v, double* out,
                     void* stream);
/* out = J^T w. */
int odil_wave_jtv_f32(const odil_wave_params* p, const float* w, float* out,
                      void* stream);
int odil_wave_jtv_f64(const odil_wave_params* p, const double* w, double* out,
                      void* stream);

/* Direct solve of J x = b by forward substitution along t (J is lower
 * triangular in C order).  Same solution as the normal equations that
 * linsolver.py:35-45 factorizes with SuperLU.  One thread block marches the
 * rows; nx <= 2048. */
int odil_wave_march_f32(const odil_wave_params* p, const float* b, float* x,
                        void* stream);
int odil_wave_march_f64(const odil_wave_params* p, const double* b, double* x,
                        void* stream);

/* One mixed-precision iterative-refinement update of a Newton step
 * (util.py:242-268 with linsolver.py:28-45): given the FP64 residual r = F(u),
 * solves J d = -r in FP32 by forward substitution and applies u += d in FP64. */
int odil_wave_refine_mixed(const odil_wave_params* p, const double* r,
                           double* u, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ODIL_GB300_H */
