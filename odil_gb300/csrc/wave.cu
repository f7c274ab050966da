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
#include <atomic>
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
// One block per tile of lg_strip; the last block adds the per-block sums.
template <typename T, int TY>
__global__ void __launch_bounds__(LG_WARPS * 32) wave_loss_grad_kernel(
    WaveDev<T> g, const T* __restrict__ u, T* __restrict__ grad, ReduceWs ws, double* loss,
    T gscale, double lscale) {
    const T lsum = lg_strip<T, TY>(g, u, grad, blockIdx.x, blockIdx.y, gscale);
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

// ---------------------------------------------------------------------------
// Vectorised fused loss + adjoint (nx a multiple of V = 16 / sizeof(T) and
// 16-byte aligned u and grad).  Same march as above, but lane l of a warp
// holds the V contiguous columns [c0 - V + V l, c0 + V l): one 16-byte load
// and one 16-byte store per lane and row, x-neighbours inside the vector from
// registers and only the two vector ends by shuffles.  Lanes 1..30 produce the
// 30 V output columns [c0, c0 + 30 V); lanes 0 and 31 are the halo.  Tiles
// that touch no boundary class evaluate the interior residual (the operation
// order of wave_f) and the interior gather with constant coefficients and
// reuse the first time difference of the previous row; the others go through
// wave_f / wave_gather cell by cell.
constexpr int LV_WARPS = 2;

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int n = 4;
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int n = 2;
};

template <typename T>
__device__ __forceinline__ void ld16(T (&v)[Vec16<T>::n], const T* p) {
    const typename Vec16<T>::type x = __ldg(reinterpret_cast<const typename Vec16<T>::type*>(p));
    if constexpr (Vec16<T>::n == 4) {
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else {
        v[0] = x.x; v[1] = x.y;
    }
}

template <typename T>
__device__ __forceinline__ void st16(T* p, const T (&v)[Vec16<T>::n]) {
    typename Vec16<T>::type x;
    if constexpr (Vec16<T>::n == 4) {
        x.x = v[0]; x.y = v[1]; x.z = v[2]; x.w = v[3];
    } else {
        x.x = v[0]; x.y = v[1];
    }
    __stcs(reinterpret_cast<typename Vec16<T>::type*>(p), x);
}

// Interior residual from the first time differences of rows (i, i-1) and
// (i-1, i-2): the operation order of wave_f's general branch.
template <typename T>
__device__ __forceinline__ T wave_f_int(const WaveDev<T>& g, T u_t_tm, T u_t_tmm, T utm, T uxm,
                                        T uxp) {
    const T u_tt = (u_t_tm - u_t_tmm) * g.inv_dt;
    const T u_xx = (uxm - T(2) * utm + uxp) * g.inv_dx2;
    return u_tt - g.c2 * u_xx;
}

// Rows of u in flight per warp: a shared-memory ring filled by cp.async
// (16 bytes per lane and row), so the prefetch depth costs no registers.
constexpr int LV_RING = 8;

template <typename T>
__device__ __forceinline__ void vload_smem(T (&v)[Vec16<T>::n], const T* p) {
    const typename Vec16<T>::type x = *reinterpret_cast<const typename Vec16<T>::type*>(p);
    if constexpr (Vec16<T>::n == 4) {
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else {
        v[0] = x.x; v[1] = x.y;
    }
}

// One warp's tile: rows [a0, a0 + TY) of the gradient at the lane's columns.
// Row q of the march (q = 0 .. TY + 3) is u row a0 - 2 + q; rows q >= 2
// produce residuals, rows q >= 4 the gradient of row q - 4 + a0.
template <typename T, int TY, bool FAST>
__device__ __forceinline__ T lg_vec_tile(const WaveDev<T>& g, const T* __restrict__ u,
                                         T* __restrict__ grad, int a0, int c0, int lane,
                                         T gscale, T* ring, T* bcs) {
    constexpr int V = Vec16<T>::n;
    constexpr int R = LV_RING;
    constexpr int NQ = TY + 4;
    static_assert((R & (R - 1)) == 0, "ring length is a power of two");
    const int nt = g.nt, nx = g.nx;
    const int cl = c0 - V + V * lane;           // first column of this lane
    const bool col_ok = cl >= 0 && cl < nx;     // nx % V == 0: all V or none
    const bool out_lane = lane >= 1 && lane <= 30 && col_ok;
    const T A = g.A, B = g.B;
    const T ctm_int = T(-2) * A + B * T(2);
    T* my = ring + lane * V;                    // this lane's slot column
    const T* src = u + (int64_t)(a0 - 2) * nx + cl;
    auto issue = [&](int q) {
        if (q < NQ) {
            const int r = a0 - 2 + q;
            T* to = my + (q & (R - 1)) * (32 * V);
            if (FAST || (r >= 0 && r < nt && col_ok)) {
                cp_async_n(to, src + (int64_t)q * nx, 16);
            } else {
#pragma unroll
                for (int e = 0; e < V; ++e) to[e] = T(0);
            }
        }
        cp_async_commit();
    };
    T u1[V], u2[V], f1[V], f2[V], ut1[V];
#pragma unroll
    for (int e = 0; e < V; ++e) u1[e] = u2[e] = f1[e] = f2[e] = ut1[e] = T(0);
    T lsum = T(0);
    // Boundary tiles: the boundary data of the tile's rows and columns are
    // staged once (left/right values per row in shared memory, initial values
    // per column in registers), so no dependent global load sits in the march.
    T iu[V], iut[V];
#pragma unroll
    for (int e = 0; e < V; ++e) iu[e] = iut[e] = T(0);
    if (!FAST) {
        for (int q = lane; q < NQ; q += 32) {
            const int r = a0 - 2 + q;
            const bool ok = r >= 1 && r <= nt;
            bcs[q] = ok ? opt_ld(g.left_u, r - 1) : T(0);
            bcs[NQ + q] = ok ? opt_ld(g.right_u, r - 1) : T(0);
        }
        if (col_ok && a0 <= 3) {
#pragma unroll
            for (int e = 0; e < V; ++e) {
                iu[e] = opt_ld(g.init_u, cl + e);
                iut[e] = opt_ld(g.init_ut, cl + e);
            }
        }
        __syncwarp();
    }
    // Residuals of row q into f0 (q >= 2); advances u1, u2, ut1.
    auto residual_row = [&](int q, const T (&u0)[V], T (&f0)[V]) {
        const int r = a0 - 2 + q;
        const T lm = __shfl_up_sync(0xffffffffu, u1[V - 1], 1);
        const T rp = __shfl_down_sync(0xffffffffu, u1[0], 1);
        if (FAST) {
            T ut0[V];
#pragma unroll
            for (int e = 0; e < V; ++e) ut0[e] = (u0[e] - u1[e]) * g.inv_dt;
#pragma unroll
            for (int e = 0; e < V; ++e) {
                const T um = e == 0 ? lm : u1[e - 1];
                const T up = e == V - 1 ? rp : u1[e + 1];
                f0[e] = wave_f_int(g, ut0[e], ut1[e], u1[e], um, up);
                ut1[e] = ut0[e];
            }
        } else {
#pragma unroll
            for (int e = 0; e < V; ++e) {
                const T um = e == 0 ? lm : u1[e - 1];
                const T up = e == V - 1 ? rp : u1[e + 1];
                const T lb = bcs[q], rb = bcs[NQ + q];
                const T a = iu[e], b = iut[e];
                f0[e] = (col_ok && r >= 0 && r < nt)
                            ? wave_f_with(
                                  g, r, cl + e, u0[e], u1[e], u2[e], um, up,
                                  [&](int) { return a; }, [&](int) { return b; },
                                  [&](int) { return lb; }, [&](int) { return rb; })
                            : T(0);
            }
        }
#pragma unroll
        for (int e = 0; e < V; ++e) {
            u2[e] = u1[e];
            u1[e] = u0[e];
        }
    };
#pragma unroll
    for (int q = 0; q < R - 1; ++q) issue(q);
    // Rows q = 0..3: no gradient yet.
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        issue(q + R - 1);
        cp_async_wait<R - 1>();
        T u0[V];
        vload_smem<T>(u0, my + q * (32 * V));
        if (q == 0 && FAST) {
#pragma unroll
            for (int e = 0; e < V; ++e) {
                u2[e] = u1[e];
                u1[e] = u0[e];
            }
        } else if (q == 1 && FAST) {
#pragma unroll
            for (int e = 0; e < V; ++e) {
                ut1[e] = (u0[e] - u1[e]) * g.inv_dt;
                u2[e] = u1[e];
                u1[e] = u0[e];
            }
        } else if (q < 2) {
            T f0[V];
            residual_row(q, u0, f0);  // rows before the tile: f unused
        } else {
            T f0[V];
            residual_row(q, u0, f0);
#pragma unroll
            for (int e = 0; e < V; ++e) {
                f2[e] = f1[e];
                f1[e] = f0[e];
            }
        }
    }
    // Rows q = 4 .. TY + 3: residual of row q, gradient of row a = r - 2.
    // Unrolled by 4 only: a whole ring turn of this body overflows the
    // instruction cache.
    T* gout = grad + (int64_t)a0 * nx + cl;
#pragma unroll 4
    for (int q = 4; q < NQ; ++q) {
        {
            issue(q + R - 1);
            cp_async_wait<R - 1>();
            T u0[V], f0[V];
            vload_smem<T>(u0, my + (q & (R - 1)) * (32 * V));
            residual_row(q, u0, f0);
            const T fl = __shfl_up_sync(0xffffffffu, f1[V - 1], 1);
            const T fr = __shfl_down_sync(0xffffffffu, f1[0], 1);
            const int a = a0 - 4 + q;
            if (out_lane && (FAST || a < nt)) {
                T gv[V];
#pragma unroll
                for (int e = 0; e < V; ++e) {
                    const T fm = e == 0 ? fl : f1[e - 1];
                    const T fp = e == V - 1 ? fr : f1[e + 1];
                    T sg;
                    if (FAST) {
                        sg = A * f2[e];
                        sg += ctm_int * f1[e];
                        sg -= B * (fp + fm);
                        sg += A * f0[e];
                    } else {
                        sg = wave_gather(g, a, cl + e, f2[e], f1[e], f0[e], fp, fm);
                    }
                    gv[e] = sg * gscale;
                    lsum += f2[e] * f2[e];
                }
                st16<T>(gout, gv);
            }
            gout += nx;
#pragma unroll
            for (int e = 0; e < V; ++e) {
                f2[e] = f1[e];
                f1[e] = f0[e];
            }
        }
    }
    cp_async_wait<0>();
    return lsum;
}

// Tile geometry of the vectorised loss: warp tiles (strip sw, row tile ty)
// cover columns [30 V sw, 30 V (sw + 1)) and rows [TY ty, TY (ty + 1)).  The
// tiles with 1 <= sw <= sw_hi and 1 <= ty <= ty_hi touch no boundary class
// (interior kernel); the rest of the grid goes to the edge kernel in tiles of
// min(TY, LV_EDGE_TY) rows, so that its short marches run in parallel.
constexpr int LV_EDGE_TY = 16;

__host__ __device__ constexpr int lv_edge_ty(int ty) { return ty < LV_EDGE_TY ? ty : LV_EDGE_TY; }

struct LvGeom {
    int nsw;           // strips across
    int sw_hi, ty_hi;  // last interior strip / interior row tile (0: none)
    int nte;           // edge row tiles down
    int lo, hi;        // edge row tiles [lo, hi] lie beside the interior
    int64_t n_int_blocks, n_edge;
    dim3 int_grid;
};

template <typename T>
LvGeom lv_geom(int nt, int nx, int ty) {
    constexpr int V = Vec16<T>::n;
    LvGeom q;
    q.nsw = (nx + 30 * V - 1) / (30 * V);
    q.sw_hi = nx >= 31 * V ? (nx - 31 * V) / (30 * V) : 0;
    q.ty_hi = nt >= ty + 2 ? (nt - ty - 2) / ty : 0;
    if (q.sw_hi < 1 || q.ty_hi < 1) q.sw_hi = q.ty_hi = 0;
    q.int_grid = dim3((q.sw_hi + LV_WARPS - 1) / LV_WARPS, q.ty_hi);
    q.n_int_blocks = (int64_t)q.int_grid.x * q.int_grid.y;
    const int ety = lv_edge_ty(ty);
    q.nte = (nt + ety - 1) / ety;
    const int per = ty / ety;
    if (q.ty_hi > 0) {
        q.lo = per;
        q.hi = (q.ty_hi + 1) * per - 1;
    } else {
        q.lo = q.nte;
        q.hi = q.nte - 1;
    }
    q.n_edge = (int64_t)q.nsw * q.nte - (int64_t)(q.hi - q.lo + 1) * q.sw_hi;
    return q;
}

// Both tile kinds in one launch: the first blocks take the boundary tiles
// (two per block, one per warp), the rest the interior tiles, so the slow
// boundary marches run beside the interior ones instead of after them.  The
// register cap of the interior path applies to the whole kernel; the
// boundary path is rare enough that its spills do not matter.
template <typename T, int TY>
__global__ void __launch_bounds__(LV_WARPS * 32, 16) wave_loss_grad_all_kernel(
    WaveDev<T> g, const T* __restrict__ u, T* __restrict__ grad, ReduceWs ws, LvGeom q,
    double* loss, T gscale, double lscale) {
    static_assert(LV_WARPS == 2, "two boundary tiles per block");
    constexpr int V = Vec16<T>::n;
    constexpr int ETY = lv_edge_ty(TY);
    __shared__ __align__(16) T ring_all[LV_WARPS][LV_RING][32 * V];
    __shared__ T bcs_all[LV_WARPS][2 * (ETY + 4)];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t neb = (q.n_edge + 1) / 2;  // boundary blocks
    const int64_t b = blockIdx.x;
    T lsum = T(0);
    if (b < neb) {
        const int64_t t = 2 * b + warp;
        if (t < q.n_edge) {
            const int64_t nfull = (int64_t)(q.nte - (q.hi - q.lo + 1)) * q.nsw;
            int sw, ty;
            if (t < nfull) {
                const int r = (int)(t / q.nsw);
                sw = (int)(t - (int64_t)r * q.nsw);
                ty = r < q.lo ? r : q.hi + 1 + (r - q.lo);
            } else {
                const int m = q.nsw - q.sw_hi;
                const int64_t k = t - nfull;
                ty = q.lo + (int)(k / m);
                const int c = (int)(k - (int64_t)(ty - q.lo) * m);
                sw = c == 0 ? 0 : q.sw_hi + c;
            }
            lsum = lg_vec_tile<T, ETY, false>(g, u, grad, ty * ETY, sw * (30 * V),
                                                     lane, gscale, &ring_all[warp][0][0],
                                                     &bcs_all[warp][0]);
        }
    } else {
        const int64_t ib = b - neb;
        const int bx = (int)(ib % q.int_grid.x), by = (int)(ib / q.int_grid.x);
        const int sw = 1 + bx * LV_WARPS + warp;
        if (sw <= q.sw_hi) {
            lsum = lg_vec_tile<T, TY, true>(g, u, grad, (1 + by) * TY, sw * (30 * V), lane,
                                            gscale, &ring_all[warp][0][0], nullptr);
        }
    }
    reduce_finish((double)lsum, b, (int64_t)gridDim.x, ws, lscale, loss);
}

// Launch plan of the fused loss + adjoint: the vectorised kernels when the
// rows allow 16-byte accesses, else the one-column-per-lane kernel.
struct LgPlan {
    dim3 grid;      // one-column-per-lane kernel
    int ty;
    bool vec;
    LvGeom geom;    // vectorised kernels
    int64_t blocks; // reduction partials
};

template <typename T>
LgPlan lg_plan(int nt, int nx, const void* u, const void* grad) {
    constexpr int V = Vec16<T>::n;
    LgPlan pl;
    pl.vec = (nx % V == 0) &&
             ((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(grad)) % 16 == 0);
    if (pl.vec) {
        const int64_t cells = (int64_t)nt * nx;
        // Taller tiles on large grids (fewer halo rows), shorter ones on
        // small grids so that enough warps run (a 1024^2 grid with 16-row
        // tiles fills 5% of the warp slots).
        pl.ty = cells >= (16 << 20) ? 64
                                    : (cells >= (4 << 20) ? 32 : (cells >= (2 << 20) ? 16 : 8));
        pl.geom = lv_geom<T>(nt, nx, pl.ty);
        pl.grid = dim3(1, pl.geom.nte);
        pl.blocks = pl.geom.n_int_blocks + (pl.geom.n_edge + 1) / 2;
    } else {
        pl.ty = lg_ty(nt, nx);
        pl.grid = lg_grid(nt, nx);
        pl.blocks = (int64_t)pl.grid.x * pl.grid.y;
    }
    return pl;
}

// Reduction blocks a caller workspace must cover for either kernel.
template <typename T>
int64_t lg_max_blocks(int nt, int nx) {
    const LgPlan a = lg_plan<T>(nt, nx, nullptr, nullptr);
    const dim3 b = lg_grid(nt, nx);
    const int64_t nb = (int64_t)b.x * b.y;
    return a.blocks > nb ? a.blocks : nb;
}

template <typename T, int TY>
void lv_launch(const LgPlan& pl, const WaveDev<T>& g, const T* u, T* grad, ReduceWs ws,
               double* loss, T gs, double ls, cudaStream_t s) {
    wave_loss_grad_all_kernel<T, TY><<<(unsigned)pl.blocks, LV_WARPS * 32, 0, s>>>(
        g, u, grad, ws, pl.geom, loss, gs, ls);
}

template <typename T>
void lg_launch_scaled(const LgPlan& pl, const WaveDev<T>& g, const T* u, T* grad, ReduceWs ws,
                      double* loss, T gs, double ls, cudaStream_t s) {
    if (pl.vec) {
        if (pl.ty == 8) {
            lv_launch<T, 8>(pl, g, u, grad, ws, loss, gs, ls, s);
        } else if (pl.ty == 16) {
            lv_launch<T, 16>(pl, g, u, grad, ws, loss, gs, ls, s);
        } else if (pl.ty == 32) {
            lv_launch<T, 32>(pl, g, u, grad, ws, loss, gs, ls, s);
        } else {
            lv_launch<T, 64>(pl, g, u, grad, ws, loss, gs, ls, s);
        }
    } else if (pl.ty == 16) {
        wave_loss_grad_kernel<T, 16><<<pl.grid, LG_WARPS * 32, 0, s>>>(g, u, grad, ws, loss, gs, ls);
    } else {
        wave_loss_grad_kernel<T, 32><<<pl.grid, LG_WARPS * 32, 0, s>>>(g, u, grad, ws, loss, gs, ls);
    }
}

template <typename T>
void lg_launch(const LgPlan& pl, const WaveDev<T>& g, const T* u, T* grad, ReduceWs ws,
               double* loss, cudaStream_t s) {
    const double n = (double)g.nt * (double)g.nx;
    lg_launch_scaled<T>(pl, g, u, grad, ws, loss, (T)(2.0 / n), 1.0 / n, s);
}

// ---------------------------------------------------------------------------
// Normal-equation pieces (the matrix J^T J of linsolver.py:35-41, never
// formed).  J^T J v: the fused adjoint above with the boundary data taken as
// zero (then F(v) = J v, F being affine in u) and the gradient scale 1, so
// one pass reads v and writes J^T J v.  diag(J^T J): per column, the sum of
// the squared coefficients of the rows that read it (the rows of
// wave_gather).
template <typename T>
__global__ void __launch_bounds__(256) wave_jtj_diag_kernel(WaveDev<T> g, T* __restrict__ out) {
    const int nt = g.nt, nx = g.nx;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (int64_t)nt * nx) return;
    const int a = (int)(k / nx), b = (int)(k - (int64_t)a * nx);
    const T cu = a == 0 ? T(1) : g.A;
    T s = cu * cu;
    if (a + 1 < nt) {
        // Row (a+1, b) and its x-neighbours read u[a, b]; where they are the
        // same row (nx <= 2) the coefficients add before squaring.
        const T ctm = (a + 1 == 1 ? -g.A : T(-2) * g.A) + g.B * k_tm<T>(b, nx);
        const int bp = (b + 1 == nx) ? 0 : b + 1;
        const int bm = (b == 0) ? nx - 1 : b - 1;
        const T cm = -g.B * k_xm<T>(bp, nx), cp = -g.B * k_xp<T>(bm, nx);
        if (nx == 1) {
            const T c = ctm + cm + cp;
            s += c * c;
        } else if (bp == bm) {
            s += ctm * ctm + (cm + cp) * (cm + cp);
        } else {
            s += ctm * ctm + cm * cm + cp * cp;
        }
    }
    if (a + 2 < nt) s += g.A * g.A;
    out[k] = s;
}

template <typename T>
int jtj_diag_impl(const odil_wave_params* p, T* out, void* stream) {
    WaveDev<T> g;
    int st = make_dev<T>(p, &g, false);
    if (st) return st;
    if (!out) return ODIL_ERR_ARG;
    const int64_t n = (int64_t)g.nt * g.nx;
    wave_jtj_diag_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(g, out);
    return launch_status();
}

template <typename T>
int64_t jtj_ws_bytes(const odil_wave_params* p) {
    WaveDev<T> g;
    if (make_dev<T>(p, &g, false)) return 0;
    // Either loss-kernel plan, + the discarded loss scalar.
    return reduce_ws_bytes(lg_max_blocks<T>(g.nt, g.nx)) + 256;
}

template <typename T>
int jtj_v_impl(const odil_wave_params* p, const T* v, T* out, void* ws, int64_t ws_bytes,
               void* stream) {
    WaveDev<T> g;
    int st = make_dev<T>(p, &g, false);  // no boundary data: F(v) = J v
    if (st) return st;
    if (!v || !out) return ODIL_ERR_ARG;
    const LgPlan pl = lg_plan<T>(g.nt, g.nx, v, out);
    if (pl.grid.y > 65535) return ODIL_ERR_SHAPE;
    const int64_t need = reduce_ws_bytes(pl.blocks) + 256;
    if (!ws || ws_bytes < need) return ODIL_ERR_WORKSPACE;
    double* loss = reinterpret_cast<double*>(static_cast<char*>(ws) + need - 256);
    lg_launch_scaled<T>(pl, g, v, out, reduce_ws(ws), loss, T(1), 0.0, as_stream(stream));
    return launch_status();
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
    if (threads > march_max_threads<T, CPT, PF>()) return ODIL_ERR_SHAPE;
    const size_t smem = march_smem_bytes<T>(nx, PF);
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
    if constexpr (march_reg<T>()) {
        // Register ring: 8 rows ahead.
        switch (march_cpt(nx)) {
            case 1: return launch_march_cfg<T, 1, 8>(g, b, x, st);
            case 2: return launch_march_cfg<T, 2, 8>(g, b, x, st);
            default: return launch_march_cfg<T, 4, 8>(g, b, x, st);
        }
    }
    // Shared-memory ring: 16 rows when it fits, else 8.
    const bool deep = march_smem_bytes<T>(nx, 16) <= 200 * 1024;
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
    const LgPlan pl = lg_plan<T>(g.nt, g.nx, u, grad);
    if (pl.grid.y > 65535) return ODIL_ERR_SHAPE;
    const int64_t nb = pl.blocks;
    if (!ws || ws_bytes < reduce_ws_bytes(nb)) return ODIL_ERR_WORKSPACE;
    lg_launch<T>(pl, g, u, grad, reduce_ws(ws), loss, as_stream(stream));
    return launch_status();
}

// Right-hand sides of the mixed Newton from zero.  Interior cells (rows >= 2,
// columns 1 .. nx-2) and boundary cells are separate launches: the interior
// one has no FP64 instruction, and the boundary one packs the boundary cells
// into full warps, so its FP64 work is not replicated across idle lanes.
//   initial:  rhs = float(-F(0)), 0 inside (a memset) and FP64 on the boundary;
//   pair:     rhs = float(-F(hi + lo)), float-pair inside.
__global__ void __launch_bounds__(256) wave_pair_interior_kernel(int nt, int nx, PairCoef k,
                                                                 const float* __restrict__ hi,
                                                                 const float* __restrict__ lo,
                                                                 float* __restrict__ rhs) {
    const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nx - 1) return;
    for (int i = 2 + blockIdx.y; i < nt; i += gridDim.y) {
        const int64_t c0 = (int64_t)i * nx + j;
        rhs[c0] = pair_interior_rhs(k, hi, lo, c0, nx);
    }
}

template <int KIND>
__global__ void __launch_bounds__(256) wave_bnd_rhs_kernel(WaveDev<double> g, PairCoef k,
                                                           const float* __restrict__ hi,
                                                           const float* __restrict__ lo,
                                                           float* __restrict__ rhs,
                                                           int64_t count) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    int i, j;
    bnd_cell(t, g.nt, g.nx, &i, &j);
    rhs[(int64_t)i * g.nx + j] = bnd_cell_rhs<KIND>(g, k, hi, lo, i, j);
}

// rhs = float(-F(0)) in one launch: the first `nbb` blocks compute the
// boundary cells (FP64, packed into full warps), the others write zeros to
// the interior (rows >= 2, columns 1 .. nx-2), where F(0) vanishes.
__global__ void __launch_bounds__(256) wave_initial_rhs_kernel(WaveDev<double> g,
                                                               float* __restrict__ rhs,
                                                               int64_t count, int nbb) {
    // The dependent march (programmatic launch) is released only after this
    // thread's writes (a thread that returns early releases at its exit).
    if ((int)blockIdx.x < nbb) {
        const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= count) return;
        int i, j;
        bnd_cell(t, g.nt, g.nx, &i, &j);
        const PairCoef k{};
        rhs[(int64_t)i * g.nx + j] = bnd_cell_rhs<0>(g, k, nullptr, nullptr, i, j);
        pdl_trigger();
        return;
    }
    const int w = g.nx - 2;
    if (g.nt <= 2 || w <= 0) return;
    const int64_t n = (int64_t)(g.nt - 2) * w;
    const int64_t stride = (int64_t)(gridDim.x - nbb) * blockDim.x;
    for (int64_t t = (int64_t)(blockIdx.x - nbb) * blockDim.x + threadIdx.x; t < n; t += stride) {
        const int64_t r = t / w;
        rhs[(r + 2) * g.nx + 1 + (t - r * w)] = 0.f;
    }
    pdl_trigger();
}

// Only the boundary cells of rhs = float(-F(0)), compactly in the bnd_cell
// order (rows 0 and 1, then columns 0 and nx-1 of each further row): the
// table a march from zero reads in place of the full right-hand side, whose
// interior is zero.  64-thread blocks spread the FP64 work over the SMs.
__global__ void __launch_bounds__(64) wave_initial_table_kernel(WaveDev<double> g,
                                                               float* __restrict__ tbl,
                                                               int64_t count) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    int i, j;
    bnd_cell(t, g.nt, g.nx, &i, &j);
    const PairCoef k{};
    tbl[t] = bnd_cell_rhs<0>(g, k, nullptr, nullptr, i, j);
    pdl_trigger();  // the dependent march is released after the write
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
    const int64_t b64 = lg_max_blocks<double>((int)p->nt, (int)p->nx);
    const int64_t b32 = lg_max_blocks<float>((int)p->nt, (int)p->nx);
    return reduce_ws_bytes(b64 > b32 ? b64 : b32);
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

ODIL_API int64_t odil_wave_jtj_workspace_bytes(const odil_wave_params* p) {
    const int64_t a = jtj_ws_bytes<float>(p), b = jtj_ws_bytes<double>(p);
    return a > b ? a : b;
}
ODIL_API int odil_wave_jtj_v_f32(const odil_wave_params* p, const float* v, float* out,
                                 void* workspace, int64_t workspace_bytes, void* stream) {
    return jtj_v_impl<float>(p, v, out, workspace, workspace_bytes, stream);
}
ODIL_API int odil_wave_jtj_v_f64(const odil_wave_params* p, const double* v, double* out,
                                 void* workspace, int64_t workspace_bytes, void* stream) {
    return jtj_v_impl<double>(p, v, out, workspace, workspace_bytes, stream);
}
ODIL_API int odil_wave_jtj_diag_f32(const odil_wave_params* p, float* out, void* stream) {
    return jtj_diag_impl<float>(p, out, stream);
}
ODIL_API int odil_wave_jtj_diag_f64(const odil_wave_params* p, double* out, void* stream) {
    return jtj_diag_impl<double>(p, out, stream);
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
    cudaStream_t s = as_stream(stream);
    const int64_t nb = bnd_count(g.nt, g.nx);
    const int nbb = (int)((nb + 255) / 256);
    const int64_t interior = (int64_t)(g.nt > 2 ? g.nt - 2 : 0) * (g.nx > 2 ? g.nx - 2 : 0);
    int64_t nzb = (interior + 255) / 256;
    if (nzb > 4 * 152) nzb = 4 * 152;  // grid-stride beyond this
    wave_initial_rhs_kernel<<<(unsigned)(nbb + nzb), 256, 0, s>>>(g, rhs, nb, nbb);
    return launch_status();
}

ODIL_API int64_t odil_wave_boundary_cells(const odil_wave_params* p) {
    if (!p || p->nt < 1 || p->nx < 1) return 0;
    return bnd_count((int)p->nt, (int)p->nx);
}

ODIL_API int odil_wave_initial_table_mixed(const odil_wave_params* p, float* tbl, void* stream) {
    WaveDev<double> g;
    int st = make_dev<double>(p, &g, true);
    if (st) return st;
    if (!tbl) return ODIL_ERR_ARG;
    const int64_t nb = bnd_count(g.nt, g.nx);
    wave_initial_table_kernel<<<(unsigned)((nb + 63) / 64), 64, 0, as_stream(stream)>>>(g, tbl,
                                                                                     nb);
    return launch_status();
}

ODIL_API int odil_wave_pair_residual_mixed(const odil_wave_params* p, const float* hi,
                                           const float* lo, float* rhs, void* stream) {
    WaveDev<double> g;
    int st = make_dev<double>(p, &g, true);
    if (st) return st;
    if (!hi || !rhs || rhs == hi || rhs == lo) return ODIL_ERR_ARG;
    if (!g.init_u || !g.init_ut || !g.left_u || !g.right_u) return ODIL_ERR_ARG;
    const PairCoef k = pair_coef((double)g.A, (double)g.B);
    cudaStream_t s = as_stream(stream);
    if (g.nt > 2 && g.nx > 2) {
        const int bx = 256;
        const int gy = g.nt - 2 < 65535 ? g.nt - 2 : 65535;
        wave_pair_interior_kernel<<<dim3((g.nx - 2 + bx - 1) / bx, gy), bx, 0, s>>>(
            g.nt, g.nx, k, hi, lo, rhs);
    }
    const int64_t nb = bnd_count(g.nt, g.nx);
    wave_bnd_rhs_kernel<1><<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(g, k, hi, lo, rhs, nb);
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
//     stream capture.  Host threads that make their first calls at once may
//     both look the address up; the cache is an atomic per device, and both
//     store the same value;
//   * the cached address belongs to the device's primary context: it does
//     not survive cudaDeviceReset (or any other teardown of that context),
//     after which this entry point must not be called in the same process.
constexpr int64_t kNoAllocBytes = 256 * 1024;
constexpr int64_t kNoAllocMaxBlocks = (kNoAllocBytes - kReduceHeader) / (int64_t)sizeof(double);
static __device__ __align__(256) unsigned char g_loss_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
std::atomic<void*> g_scratch_ptr[kMaxDevices];

// Device address of g_loss_scratch on the current device (set-up on first use).
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return ODIL_ERR_LAUNCH;
    void* ptr = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!ptr) {
        if (cudaGetSymbolAddress(&ptr, g_loss_scratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return ODIL_ERR_LAUNCH;
        }
        g_scratch_ptr[dev].store(ptr, std::memory_order_release);
    }
    *out = ptr;
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
    const LgPlan pl = lg_plan<float>(g.nt, g.nx, u, grad);
    if (pl.grid.y > 65535) return ODIL_ERR_SHAPE;
    const int64_t nb = pl.blocks;
    if (nb > kNoAllocMaxBlocks) return ODIL_ERR_WORKSPACE;
    void* ws = nullptr;
    st = scratch_address(&ws);
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (cudaMemsetAsync(ws, 0, sizeof(unsigned), s) != cudaSuccess) return ODIL_ERR_LAUNCH;
    lg_launch<float>(pl, g, u, grad, reduce_ws(ws), loss, s);
    return launch_status();
}
