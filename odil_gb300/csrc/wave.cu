// 1D wave operator on the (t, x) space-time grid: residual, fused loss+adjoint
// gradient, matrix-free J v / J^T w, and the forward-substitution direct solve.
//
// Reference: wave.py:67-122 (operator_fd), util_op.py:508-563 (roll semantics
// of Context.field), util_op.py:585-614 (per-shift Jacobian), util_op.py:
// 627-654 (loss), linsolver.py:28-45 (Newton linear solve).
//
// Jacobian in stencil form.  Row (i, j) of J couples to five "slots":
//   u = (i, j), tm = (i-1, j), tmm = (i-2, j), xm = (i-1, j-1), xp = (i-1, j+1)
// (indices periodic, as tf.roll).  With A = 1/dt^2, B = c^2/dx^2:
//   row 0:   c_u = 1, all other slots 0
//   row >=1: c_u = A, c_tm = -(1 or 2) A + B k_tm, c_tmm = (0 or 1) A,
//            c_xm = -B k_xm, c_xp = -B k_xp
// where (k_tm, k_xm, k_xp) depend on the column class through the quadratic
// extrapolation of the x-halo: interior (2, 1, 1), j = 0 (4, 0, 4/3),
// j = nx-1 (4, 4/3, 0), nx = 1 (20/3, 0, 4/9).  These are the derivatives
// tf.GradientTape returns for each rolled argument, including the zero
// gradient through the branch tf.where did not take.
#include "wave_dev.cuh"

namespace odil {
namespace {
using namespace wavedev;

// ---------------------------------------------------------------------------
// Residual / J v: one thread per cell, stencil values through the read-only
// cache (each u is reused by 5 neighbouring threads; DRAM sees it once).
template <typename T>
__global__ void __launch_bounds__(256) wave_residual_kernel(WaveDev<T> g, const T* __restrict__ u,
                                                            T* __restrict__ f) {
    const int nx = g.nx;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nx) return;
    for (int i = blockIdx.y; i < g.nt; i += gridDim.y) {
        const T uc = __ldg(u + (int64_t)i * nx + j);
        T utm = 0, utmm = 0, uxm = 0, uxp = 0;
        if (i >= 1) {
            const T* r1 = u + (int64_t)(i - 1) * nx;
            utm = __ldg(r1 + j);
            uxm = __ldg(r1 + (j == 0 ? nx - 1 : j - 1));
            uxp = __ldg(r1 + (j + 1 == nx ? 0 : j + 1));
        }
        if (i >= 2) utmm = __ldg(u + (int64_t)(i - 2) * nx + j);
        f[(int64_t)i * nx + j] = wave_f(g, i, j, uc, utm, utmm, uxm, uxp);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) wave_jtv_kernel(WaveDev<T> g, const T* __restrict__ w,
                                                       T* __restrict__ out) {
    const int nx = g.nx, nt = g.nt;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nx) return;
    const int bp = (b + 1 == nx) ? 0 : b + 1;
    const int bm = (b == 0) ? nx - 1 : b - 1;
    for (int a = blockIdx.y; a < nt; a += gridDim.y) {
        const T fu = __ldg(w + (int64_t)a * nx + b);
        T ftm = 0, fxm = 0, fxp = 0, ftmm = 0;
        if (a + 1 < nt) {
            const T* r1 = w + (int64_t)(a + 1) * nx;
            ftm = __ldg(r1 + b);
            fxm = __ldg(r1 + bp);
            fxp = __ldg(r1 + bm);
        }
        if (a + 2 < nt) ftmm = __ldg(w + (int64_t)(a + 2) * nx + b);
        out[(int64_t)a * nx + b] = wave_gather(g, a, b, fu, ftm, ftmm, fxm, fxp);
    }
}

template <typename T>
void grid_rows(const WaveDev<T>& g, dim3* grid, dim3* block) {
    const int bx = g.nx >= 256 ? 256 : ((g.nx + 31) / 32) * 32;
    *block = dim3(bx);
    int gy = g.nt < 65535 ? g.nt : 65535;
    *grid = dim3((g.nx + bx - 1) / bx, gy);
}

// ---------------------------------------------------------------------------
// Fused loss + adjoint gradient, one warp per 32-column strip marching down a
// tile of rows.  Lane l holds column c0 - 1 + l; lanes 1..30 produce outputs,
// lanes 0 and 31 are the halo.  Per row the warp loads u once (coalesced; the
// two halo lanes load one extra neighbour), gets the x-neighbours of the
// previous row by shuffles, evaluates the residual of the row (kept in
// registers, never stored), and gathers J^T f for the row two above:
//   g(a, b) = sum over the rows (a, b), (a+1, b), (a+2, b), (a+1, b-1),
//             (a+1, b+1) that read u(a, b), of coefficient * f.
// Warps whose rows and columns avoid the boundary classes use the constant
// interior coefficients; the others use the general class functions.
constexpr int LG_WARPS = 4;
constexpr int LG_OUT = 30;  // output columns per warp

template <typename T, int TY>
__global__ void __launch_bounds__(LG_WARPS * 32) wave_loss_grad_kernel(
    WaveDev<T> g, const T* __restrict__ u, T* __restrict__ grad, ReduceWs ws, double* loss,
    T gscale, double lscale) {
    const int nt = g.nt, nx = g.nx;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int c0 = (blockIdx.x * LG_WARPS + warp) * LG_OUT;  // first output column
    const int a0 = blockIdx.y * TY;
    const int col = c0 - 1 + lane;
    const bool out_lane = lane >= 1 && lane <= LG_OUT && col < nx;
    const int colw = wrapn(col, nx);
    const int colm = wrapn(col - 1, nx);  // lane 0's extra load
    const int colp = wrapn(col + 1, nx);  // lane 31's extra load
    const bool fast = (c0 >= 2) && (c0 + LG_OUT + 2 <= nx) && (a0 >= 1) && (a0 + TY + 2 < nt);
    const T A = g.A, B = g.B;
    const T ctm_int = T(-2) * A + T(2) * B;

    T u1 = 0, u2 = 0, e1 = 0;   // u rows r-1, r-2 at this lane; e1: lane-0/31 extra of row r-1
    T f1 = 0, f2 = 0;           // f rows r-1, r-2
    T f1m = 0, f1p = 0;         // f row r-1 at col-1, col+1
    // Per-thread loss partial in the working precision (at most TY terms);
    // FP64 only across threads and blocks, off the per-cell path.
    T lsum = T(0);
    // Rows stream in chunks of LGQ; the loads of chunk c+1 are issued before
    // chunk c is processed, so each warp keeps up to 2 LGQ row loads in
    // flight while the shuffle chain of the march runs.
    constexpr int LGQ = 4;
    static_assert((TY + 4) % LGQ == 0, "row chunking");
    T uq[LGQ], eq[LGQ], un[LGQ], en[LGQ];
    auto load_chunk = [&](int q0, T* uu, T* ee) {
#pragma unroll
        for (int j = 0; j < LGQ; ++j) {
            const int r = a0 - 2 + q0 + j;
            uu[j] = T(0);
            ee[j] = T(0);
            if (q0 + j < TY + 4 && r >= 0 && r < nt) {
                const T* row = u + (int64_t)r * nx;
                uu[j] = __ldg(row + colw);
                if (lane == 0) ee[j] = __ldg(row + colm);
                if (lane == 31) ee[j] = __ldg(row + colp);
            }
        }
    };
    load_chunk(0, uq, eq);
    for (int q0 = 0; q0 < TY + 4; q0 += LGQ) {
        load_chunk(q0 + LGQ, un, en);
#pragma unroll
        for (int j = 0; j < LGQ; ++j) {
            const int q = q0 + j;
            const int r = a0 - 2 + q;
            const T u0 = uq[j], e0 = eq[j];
            // x-neighbours of row r-1 at this lane.
            T um = __shfl_up_sync(0xffffffffu, u1, 1);
            T up = __shfl_down_sync(0xffffffffu, u1, 1);
            if (lane == 0) um = e1;
            if (lane == 31) up = e1;
            if (q >= 2) {
                T f0 = T(0);
                if (r < nt) f0 = wave_f(g, r, colw, u0, u1, u2, um, up);
                // Gradient of row a = r - 2 (f rows a, a+1 with neighbours, a+2).
                if (q >= 4 && out_lane) {
                    const int a = r - 2;
                    if (a < nt) {
                        T gs;
                        if (fast) {
                            gs = A * (f2 + f0) + ctm_int * f1 - B * (f1p + f1m);
                        } else {
                            gs = wave_gather(g, a, col, f2, f1, f0, f1p, f1m);
                        }
                        grad[(int64_t)a * nx + col] = gs * gscale;
                        lsum += f2 * f2;
                    }
                }
                f2 = f1;
                f1 = f0;
                f1m = __shfl_up_sync(0xffffffffu, f0, 1);
                f1p = __shfl_down_sync(0xffffffffu, f0, 1);
            }
            u2 = u1;
            u1 = u0;
            e1 = e0;
        }
#pragma unroll
        for (int j = 0; j < LGQ; ++j) {
            uq[j] = un[j];
            eq[j] = en[j];
        }
    }
    const int64_t bid = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
    const int64_t nb = (int64_t)gridDim.x * gridDim.y;
    reduce_finish((double)lsum, bid, nb, ws, lscale, loss);
}

inline int lg_ty(int nt, int nx) { return (int64_t)nt * nx < (4 << 20) ? 16 : 32; }

inline dim3 lg_grid(int nt, int nx) {
    const int ty = lg_ty(nt, nx);
    const int cols = LG_WARPS * LG_OUT;
    return dim3((nx + cols - 1) / cols, (nt + ty - 1) / ty);
}

// Columns per thread for a row of nx cells (at most 1024 threads).
inline int march_cpt(int nx) {
    if (nx <= 128) return 1;
    if (nx <= 1024) return 2;
    return 4;
}

template <typename T, int CPT, int PF>
int launch_march_cfg(const WaveDev<T>& g, const T* b, T* x, cudaStream_t st) {
    const int nx = g.nx;
    const bool vec = (nx % CPT == 0) &&
                     ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(x)) %
                      (CPT * sizeof(T))) == 0;
    int threads = (nx + CPT - 1) / CPT;
    threads = ((threads + 31) / 32) * 32;
    if (threads > 1024) return ODIL_ERR_SHAPE;
    const size_t smem = (2 + PF) * (size_t)nx * sizeof(T);
    auto go = [&](auto kern) {
        ensure_dynamic_smem(reinterpret_cast<const void*>(kern), smem);
        kern<<<1, threads, smem, st>>>(g, b, x);
    };
    if (vec) {
        go(wave_march_kernel<T, CPT, PF, true>);
    } else {
        go(wave_march_kernel<T, CPT, PF, false>);
    }
    return launch_status();
}

template <typename T>
int launch_march(const WaveDev<T>& g, const T* b, T* x, cudaStream_t st) {
    const int nx = g.nx;
    if (nx > 2048) return ODIL_ERR_SHAPE;
    // Ring depth: 16 rows when it fits in shared memory, else 8.
    const bool deep = (2 + 16) * (size_t)nx * sizeof(T) <= 200 * 1024;
    switch (march_cpt(nx)) {
        case 1: return deep ? launch_march_cfg<T, 1, 16>(g, b, x, st)
                            : launch_march_cfg<T, 1, 8>(g, b, x, st);
        case 2: return deep ? launch_march_cfg<T, 2, 16>(g, b, x, st)
                            : launch_march_cfg<T, 2, 8>(g, b, x, st);
        default: return deep ? launch_march_cfg<T, 4, 16>(g, b, x, st)
                             : launch_march_cfg<T, 4, 8>(g, b, x, st);
    }
}

// ---------------------------------------------------------------------------
// One fully parallel FP64 step of mixed-precision Newton: u_out = u + d (d is
// the FP32 correction of the previous march, or absent), r = F(u_out) in FP64,
// rhs = float(-r) for the next FP32 march, optionally sum(r^2) in FP64.  The
// stencil reads u + d at the five neighbours itself, so u_out must not alias u.
template <bool HAS_D, bool NORM>
__global__ void __launch_bounds__(256) wave_update_residual_kernel(
    WaveDev<double> g, const double* __restrict__ u, const float* __restrict__ d,
    double* __restrict__ uout, float* __restrict__ rhs, ReduceWs ws, double* rnorm2) {
    const int nx = g.nx, nt = g.nt;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (j < nx) {
        const int jm = j == 0 ? nx - 1 : j - 1;
        const int jp = j + 1 == nx ? 0 : j + 1;
        for (int i = blockIdx.y; i < nt; i += gridDim.y) {
            auto val = [&](int ii, int jj) -> double {
                const int64_t k = (int64_t)ii * nx + jj;
                double v = __ldg(u + k);
                if constexpr (HAS_D) v += (double)__ldg(d + k);
                return v;
            };
            const double uc = val(i, j);
            double utm = 0, utmm = 0, uxm = 0, uxp = 0;
            if (i >= 1) {
                utm = val(i - 1, j);
                uxm = val(i - 1, jm);
                uxp = val(i - 1, jp);
            }
            if (i >= 2) utmm = val(i - 2, j);
            const double f = wave_f(g, i, j, uc, utm, utmm, uxm, uxp);
            const int64_t k = (int64_t)i * nx + j;
            if constexpr (HAS_D) uout[k] = uc;
            rhs[k] = (float)(-f);
            if constexpr (NORM) acc += f * f;
        }
    }
    if constexpr (NORM) {
        const int64_t bid = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
        reduce_finish(acc, bid, (int64_t)gridDim.x * gridDim.y, ws, 1.0, rnorm2);
    }
}

inline dim3 ur_grid(int nt, int nx, dim3* block) {
    const int bx = nx >= 256 ? 256 : ((nx + 31) / 32) * 32;
    *block = dim3(bx);
    const int gy = nt < 4096 ? nt : 4096;
    return dim3((nx + bx - 1) / bx, gy);
}

template <typename T>
int residual_impl(const odil_wave_params* p, const T* u, T* f, void* stream, bool with_bc) {
    WaveDev<T> g;
    int st = make_dev<T>(p, &g, with_bc);
    if (st) return st;
    if (!u || !f) return ODIL_ERR_ARG;
    dim3 grid, block;
    grid_rows(g, &grid, &block);
    wave_residual_kernel<T><<<grid, block, 0, as_stream(stream)>>>(g, u, f);
    return launch_status();
}

template <typename T>
int jtv_impl(const odil_wave_params* p, const T* w, T* out, void* stream) {
    WaveDev<T> g;
    int st = make_dev<T>(p, &g, false);
    if (st) return st;
    if (!w || !out) return ODIL_ERR_ARG;
    dim3 grid, block;
    grid_rows(g, &grid, &block);
    wave_jtv_kernel<T><<<grid, block, 0, as_stream(stream)>>>(g, w, out);
    return launch_status();
}

template <typename T>
int loss_grad_impl(const odil_wave_params* p, const T* u, T* grad, double* loss, void* ws,
                   int64_t ws_bytes, void* stream) {
    WaveDev<T> g;
    int st = make_dev<T>(p, &g, true);
    if (st) return st;
    if (!u || !grad || !loss) return ODIL_ERR_ARG;
    const dim3 grid = lg_grid(g.nt, g.nx);
    if (grid.y > 65535) return ODIL_ERR_SHAPE;
    const int64_t nb = (int64_t)grid.x * grid.y;
    if (!ws || ws_bytes < reduce_ws_bytes(nb)) return ODIL_ERR_WORKSPACE;
    const double n = (double)g.nt * (double)g.nx;
    if (lg_ty(g.nt, g.nx) == 16) {
        wave_loss_grad_kernel<T, 16><<<grid, LG_WARPS * 32, 0, as_stream(stream)>>>(
            g, u, grad, reduce_ws(ws), loss, (T)(2.0 / n), 1.0 / n);
    } else {
        wave_loss_grad_kernel<T, 32><<<grid, LG_WARPS * 32, 0, as_stream(stream)>>>(
            g, u, grad, reduce_ws(ws), loss, (T)(2.0 / n), 1.0 / n);
    }
    return launch_status();
}

// rhs = float(-F(0)) for the first mixed Newton epoch from u = 0: the
// residual of the zero field is nonzero only where boundary data enter (rows
// 0 and 1, columns 0 and nx-1), so only those cells do FP64 work.
__global__ void __launch_bounds__(256) wave_initial_rhs_kernel(WaveDev<double> g,
                                                               float* __restrict__ rhs) {
    const int nx = g.nx;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nx) return;
    for (int i = blockIdx.y; i < g.nt; i += gridDim.y) {
        float v = 0.f;
        if (i <= 1 || j == 0 || j == nx - 1) v = (float)(-wave_f(g, i, j, 0.0, 0.0, 0.0, 0.0, 0.0));
        rhs[(int64_t)i * nx + j] = v;
    }
}

template <int CPT, int PF>
int launch_march_shape(const WaveDev<float>& g, const float* b, float* x, cudaStream_t st) {
    return launch_march_cfg<float, CPT, PF>(g, b, x, st);
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int64_t odil_wave_workspace_bytes(const odil_wave_params* p) {
    if (!p || p->nt < 1 || p->nx < 1) return 0;
    const dim3 grid = lg_grid((int)p->nt, (int)p->nx);
    return reduce_ws_bytes((int64_t)grid.x * grid.y);
}

ODIL_API int odil_wave_residual_f32(const odil_wave_params* p, const float* u, float* f,
                                    void* stream) {
    return residual_impl<float>(p, u, f, stream, true);
}
ODIL_API int odil_wave_residual_f64(const odil_wave_params* p, const double* u, double* f,
                                    void* stream) {
    return residual_impl<double>(p, u, f, stream, true);
}
ODIL_API int odil_wave_jv_f32(const odil_wave_params* p, const float* v, float* out,
                              void* stream) {
    return residual_impl<float>(p, v, out, stream, false);
}
ODIL_API int odil_wave_jv_f64(const odil_wave_params* p, const double* v, double* out,
                              void* stream) {
    return residual_impl<double>(p, v, out, stream, false);
}
ODIL_API int odil_wave_jtv_f32(const odil_wave_params* p, const float* w, float* out,
                               void* stream) {
    return jtv_impl<float>(p, w, out, stream);
}
ODIL_API int odil_wave_jtv_f64(const odil_wave_params* p, const double* w, double* out,
                               void* stream) {
    return jtv_impl<double>(p, w, out, stream);
}
ODIL_API int odil_wave_loss_grad_f32(const odil_wave_params* p, const float* u, float* grad,
                                     double* loss, void* workspace, int64_t workspace_bytes,
                                     void* stream) {
    return loss_grad_impl<float>(p, u, grad, loss, workspace, workspace_bytes, stream);
}
ODIL_API int odil_wave_loss_grad_f64(const odil_wave_params* p, const double* u, double* grad,
                                     double* loss, void* workspace, int64_t workspace_bytes,
                                     void* stream) {
    return loss_grad_impl<double>(p, u, grad, loss, workspace, workspace_bytes, stream);
}
ODIL_API int odil_wave_march_f32(const odil_wave_params* p, const float* b, float* x,
                                 void* stream) {
    WaveDev<float> g;
    int st = make_dev<float>(p, &g, false);
    if (st) return st;
    if (!b || !x) return ODIL_ERR_ARG;
    return launch_march<float>(g, b, x, as_stream(stream));
}
ODIL_API int odil_wave_march_f64(const odil_wave_params* p, const double* b, double* x,
                                 void* stream) {
    WaveDev<double> g;
    int st = make_dev<double>(p, &g, false);
    if (st) return st;
    if (!b || !x) return ODIL_ERR_ARG;
    return launch_march<double>(g, b, x, as_stream(stream));
}
ODIL_API int64_t odil_wave_update_residual_workspace_bytes(const odil_wave_params* p) {
    if (!p || p->nt < 1 || p->nx < 1) return 0;
    dim3 block;
    const dim3 grid = ur_grid((int)p->nt, (int)p->nx, &block);
    return reduce_ws_bytes((int64_t)grid.x * grid.y);
}
ODIL_API int odil_wave_update_residual_mixed(const odil_wave_params* p, const double* u,
                                             const float* d, double* u_out, float* rhs,
                                             double* rnorm2, void* workspace,
                                             int64_t workspace_bytes, void* stream) {
    WaveDev<double> g;
    int st = make_dev<double>(p, &g, true);
    if (st) return st;
    if (!u || !rhs || (d && !u_out)) return ODIL_ERR_ARG;
    if (d && u_out == u) return ODIL_ERR_ARG;
    dim3 block;
    const dim3 grid = ur_grid(g.nt, g.nx, &block);
    ReduceWs ws = {};
    if (rnorm2) {
        if (!workspace || workspace_bytes < reduce_ws_bytes((int64_t)grid.x * grid.y))
            return ODIL_ERR_WORKSPACE;
        ws = reduce_ws(workspace);
    }
    cudaStream_t s = as_stream(stream);
    if (d) {
        if (rnorm2)
            wave_update_residual_kernel<true, true><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
        else
            wave_update_residual_kernel<true, false><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
    } else {
        if (rnorm2)
            wave_update_residual_kernel<false, true><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
        else
            wave_update_residual_kernel<false, false><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
    }
    return launch_status();
}

ODIL_API int odil_wave_initial_rhs_mixed(const odil_wave_params* p, float* rhs, void* stream) {
    WaveDev<double> g;
    int st = make_dev<double>(p, &g, true);
    if (st) return st;
    if (!rhs) return ODIL_ERR_ARG;
    dim3 grid, block;
    grid_rows(g, &grid, &block);
    wave_initial_rhs_kernel<<<grid, block, 0, as_stream(stream)>>>(g, rhs);
    return launch_status();
}

ODIL_API int odil_wave_march_shape_f32(const odil_wave_params* p, const float* b, float* x,
                                       int32_t cpt, int32_t pf, void* stream) {
    WaveDev<float> g;
    int st = make_dev<float>(p, &g, false);
    if (st) return st;
    if (!b || !x) return ODIL_ERR_ARG;
    if ((int64_t)g.nx > 1024 * (int64_t)cpt) return ODIL_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    switch (cpt * 100 + pf) {
        case 108: return launch_march_shape<1, 8>(g, b, x, s);
        case 116: return launch_march_shape<1, 16>(g, b, x, s);
        case 208: return launch_march_shape<2, 8>(g, b, x, s);
        case 216: return launch_march_shape<2, 16>(g, b, x, s);
        case 408: return launch_march_shape<4, 8>(g, b, x, s);
        case 416: return launch_march_shape<4, 16>(g, b, x, s);
        case 808: return launch_march_shape<8, 8>(g, b, x, s);
        case 816: return launch_march_shape<8, 16>(g, b, x, s);
        default: return ODIL_ERR_SHAPE;
    }
}

// ---------------------------------------------------------------------------
// Allocation-free variant of odil_wave_loss_grad_f32.
//
// Some callers cannot allocate device memory at all: a host framework whose
// memory pool is sized and sealed at start-up, a real-time loop with a fixed
// memory budget, a plugin whose process hands it no allocator.  For them the reduction scratch of the fused loss lives in
// this file-scope device array instead of a caller workspace.  Every GPU that
// loads the library holds these 256 KiB until the process exits.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxBlocks reduction blocks (grid of the fused kernel,
//     odil_wave_loss_grad_noalloc_max_blocks()); larger grids are rejected
//     with ODIL_ERR_WORKSPACE before anything is launched;
//   * every call shares the one array, which keeps the previous call's
//     partial sums: the counter that must start at zero is cleared on the
//     stream before each launch, and calls that overlap on the GPU (other
//     streams, other host threads) race on the array;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress and caches it; make that first call before any
//     stream capture.
constexpr int64_t kNoAllocBytes = 256 * 1024;
constexpr int64_t kNoAllocMaxBlocks = (kNoAllocBytes - kReduceHeader) / (int64_t)sizeof(double);
static __device__ __align__(256) unsigned char g_loss_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_loss_scratch on the current device (set-up on first use).
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return ODIL_ERR_LAUNCH;
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_loss_scratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return ODIL_ERR_LAUNCH;
        }
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return ODIL_OK;
}
}  // namespace

ODIL_API int64_t odil_wave_loss_grad_noalloc_max_blocks(void) { return kNoAllocMaxBlocks; }

ODIL_API int odil_wave_loss_grad_f32_noalloc(const odil_wave_params* p, const float* u,
                                             float* grad, double* loss, void* stream) {
    WaveDev<float> g;
    int st = make_dev<float>(p, &g, true);
    if (st) return st;
    if (!u || !grad || !loss) return ODIL_ERR_ARG;
    const dim3 grid = lg_grid(g.nt, g.nx);
    if (grid.y > 65535) return ODIL_ERR_SHAPE;
    const int64_t nb = (int64_t)grid.x * grid.y;
    if (nb > kNoAllocMaxBlocks) return ODIL_ERR_WORKSPACE;
    void* ws = nullptr;
    st = scratch_address(&ws);
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (cudaMemsetAsync(ws, 0, sizeof(unsigned), s) != cudaSuccess) return ODIL_ERR_LAUNCH;
    const double n = (double)g.nt * (double)g.nx;
    if (lg_ty(g.nt, g.nx) == 16) {
        wave_loss_grad_kernel<float, 16><<<grid, LG_WARPS * 32, 0, s>>>(
            g, u, grad, reduce_ws(ws), loss, (float)(2.0 / n), 1.0 / n);
    } else {
        wave_loss_grad_kernel<float, 32><<<grid, LG_WARPS * 32, 0, s>>>(
            g, u, grad, reduce_ws(ws), loss, (float)(2.0 / n), 1.0 / n);
    }
    return launch_status();
}
