// 2D linear advection on the (t, x, y) space-time grid, periodic in x and y,
// first-order upwind in space, backward difference in t:
//   f = (p - ptm)/dt + ax p_x + ay p_y,   ptm = p[i-1], row 0: ptm = p_init,
//   p_x = (p - p[x-1])/dx if ax > 0 else (p[x+1] - p)/dx   (same in y).
// Reference: advection_2d.py:103-223 (operator, direct problem, --periodic 1)
// with the velocity frozen and constant (the benchmark instance).
//
// Also the matrix-free geometric multigrid on the same operator (coarse
// levels rediscretise it with doubled steps): damped Jacobi, residual,
// full-weighting restriction (the transpose of trilinear prolongation / 8),
// trilinear prolongation-add, and a dense FP64 coarsest-level solve.
#include <initializer_list>

#include "common.cuh"

namespace odil {
namespace {

template <typename T>
struct AdvDev {
    int nt, nx, ny;
    T inv_dt, inv_dx, inv_dy, ax, ay;
    T D;                      // diagonal: 1/dt + |ax|/dx + |ay|/dy
    T inv_D;                  // 1/D (the Jacobi sweep multiplies)
    bool axpos, aypos;
    const T* p_init;          // [nx * ny] or null (zero)
};

template <typename T>
int make_adv(const odil_advect_params* p, AdvDev<T>* g, bool with_init) {
    if (!p) return ODIL_ERR_ARG;
    if (p->nt < 1 || p->nx < 1 || p->ny < 1 || p->nt > 65535 || p->nx > 65535 ||
        p->ny > (1 << 30) || p->nt * p->nx * p->ny > (int64_t(1) << 31) - 1)
        return ODIL_ERR_SHAPE;
    if (!(p->dt > 0) || !(p->dx > 0) || !(p->dy > 0)) return ODIL_ERR_ARG;
    g->nt = (int)p->nt;
    g->nx = (int)p->nx;
    g->ny = (int)p->ny;
    g->inv_dt = (T)(1.0 / p->dt);
    g->inv_dx = (T)(1.0 / p->dx);
    g->inv_dy = (T)(1.0 / p->dy);
    g->ax = (T)p->ax;
    g->ay = (T)p->ay;
    g->D = (T)(1.0 / p->dt + fabs(p->ax) / p->dx + fabs(p->ay) / p->dy);
    g->inv_D = (T)(1.0 / (1.0 / p->dt + fabs(p->ax) / p->dx + fabs(p->ay) / p->dy));
    g->axpos = p->ax > 0;
    g->aypos = p->ay > 0;
    g->p_init = with_init ? (const T*)p->p_init : nullptr;
    return ODIL_OK;
}

struct Cell {
    int i, x, y;
    int64_t k;
};

template <typename T>
__device__ __forceinline__ bool cell_of(const AdvDev<T>& g, Cell* c) {
    c->y = blockIdx.x * blockDim.x + threadIdx.x;
    c->x = blockIdx.y;
    c->i = blockIdx.z;
    c->k = ((int64_t)c->i * g.nx + c->x) * g.ny + c->y;
    return c->y < g.ny;
}

inline void adv_launch_dims(int nt, int nx, int ny, dim3* grid, dim3* block) {
    const int bx = ny >= 256 ? 256 : ((ny + 31) / 32) * 32;
    *block = dim3(bx);
    *grid = dim3((ny + bx - 1) / bx, nx, nt);
}

// Residual of a cell from its upwind stencil (operation order of
// advection_2d.py:129-138, 217-220).  ptm is the previous-time value (already
// replaced by p_init on row 0 by the caller).
template <typename T>
__device__ __forceinline__ T adv_f(const AdvDev<T>& g, T p, T ptm, T pxm, T pxp, T pym, T pyp) {
    const T p_t = (p - ptm) * g.inv_dt;
    const T p_x = g.axpos ? (p - pxm) * g.inv_dx : (pxp - p) * g.inv_dx;
    const T p_y = g.aypos ? (p - pym) * g.inv_dy : (pyp - p) * g.inv_dy;
    return p_t + g.ax * p_x + g.ay * p_y;
}

// Loads the stencil of cell c from `u` (+ optional FP32 correction d) and
// returns the residual; with_init = false gives the linear part J v.
template <typename T, typename TD>
__device__ __forceinline__ T adv_eval(const AdvDev<T>& g, const Cell& c, const T* __restrict__ u,
                                      const TD* __restrict__ d, T* center) {
    const int nx = g.nx, ny = g.ny;
    auto val = [&](int64_t k) -> T {
        T v = __ldg(u + k);
        if (d) v += (T)__ldg(d + k);
        return v;
    };
    const T p = val(c.k);
    *center = p;
    T ptm;
    if (c.i == 0) {
        ptm = g.p_init ? __ldg(g.p_init + (int64_t)c.x * ny + c.y) : T(0);
    } else {
        ptm = val(c.k - (int64_t)nx * ny);
    }
    const int64_t rowk = c.k - c.y;                    // (i, x, 0)
    const int64_t slab = c.k - (int64_t)c.x * ny - c.y;  // (i, 0, 0)
    T pxm = 0, pxp = 0, pym = 0, pyp = 0;
    if (g.axpos) {
        pxm = val(slab + (int64_t)(c.x == 0 ? nx - 1 : c.x - 1) * ny + c.y);
    } else {
        pxp = val(slab + (int64_t)(c.x + 1 == nx ? 0 : c.x + 1) * ny + c.y);
    }
    if (g.aypos) {
        pym = val(rowk + (c.y == 0 ? ny - 1 : c.y - 1));
    } else {
        pyp = val(rowk + (c.y + 1 == ny ? 0 : c.y + 1));
    }
    return adv_f(g, p, ptm, pxm, pxp, pym, pyp);
}

template <typename T>
__global__ void __launch_bounds__(256) adv_residual_kernel(AdvDev<T> g, const T* __restrict__ u,
                                                           T* __restrict__ f) {
    Cell c;
    if (!cell_of(g, &c)) return;
    T center;
    f[c.k] = adv_eval<T, float>(g, c, u, nullptr, &center);
}

// J^T w at (i, x, y): the rows that read p(i, x, y) are (i, x, y) [D],
// (i+1, x, y) [-1/dt], the downwind x-neighbour [-|ax|/dx] and y-neighbour.
template <typename T>
__device__ __forceinline__ T adv_gather(const AdvDev<T>& g, const Cell& c, const T* __restrict__ w) {
    const int nx = g.nx, ny = g.ny;
    T s = g.D * __ldg(w + c.k);
    if (c.i + 1 < g.nt) s -= g.inv_dt * __ldg(w + c.k + (int64_t)nx * ny);
    const int64_t slab = c.k - (int64_t)c.x * ny - c.y;
    const int64_t rowk = c.k - c.y;
    if (g.axpos) {
        s -= g.ax * g.inv_dx * __ldg(w + slab + (int64_t)(c.x + 1 == nx ? 0 : c.x + 1) * ny + c.y);
    } else {
        s += g.ax * g.inv_dx * __ldg(w + slab + (int64_t)(c.x == 0 ? nx - 1 : c.x - 1) * ny + c.y);
    }
    if (g.aypos) {
        s -= g.ay * g.inv_dy * __ldg(w + rowk + (c.y + 1 == ny ? 0 : c.y + 1));
    } else {
        s += g.ay * g.inv_dy * __ldg(w + rowk + (c.y == 0 ? ny - 1 : c.y - 1));
    }
    return s;
}

template <typename T>
__global__ void __launch_bounds__(256) adv_jtv_kernel(AdvDev<T> g, const T* __restrict__ w,
                                                      T* __restrict__ out) {
    Cell c;
    if (!cell_of(g, &c)) return;
    out[c.k] = adv_gather(g, c, w);
}

// Fused loss + adjoint: the residuals of the (at most) four rows that read
// p(i, x, y) are recomputed in the thread; nothing is stored but the gradient.
template <typename T>
__global__ void __launch_bounds__(256) adv_loss_grad_kernel(AdvDev<T> g, const T* __restrict__ u,
                                                            T* __restrict__ grad, ReduceWs ws,
                                                            double* loss, T gscale,
                                                            double lscale) {
    Cell c;
    double acc = 0.0;
    if (cell_of(g, &c)) {
        const int nx = g.nx, ny = g.ny;
        T center;
        const T f0 = adv_eval<T, float>(g, c, u, nullptr, &center);
        acc = (double)f0 * (double)f0;
        T s = g.D * f0;
        if (c.i + 1 < g.nt) {
            Cell n = c;
            n.i += 1;
            n.k += (int64_t)nx * ny;
            s -= g.inv_dt * adv_eval<T, float>(g, n, u, nullptr, &center);
        }
        {
            Cell n = c;
            const int xs = g.axpos ? (c.x + 1 == nx ? 0 : c.x + 1) : (c.x == 0 ? nx - 1 : c.x - 1);
            n.k += (int64_t)(xs - c.x) * ny;
            n.x = xs;
            const T fn = adv_eval<T, float>(g, n, u, nullptr, &center);
            s += (g.axpos ? -g.ax : g.ax) * g.inv_dx * fn;
        }
        {
            Cell n = c;
            const int ys = g.aypos ? (c.y + 1 == ny ? 0 : c.y + 1) : (c.y == 0 ? ny - 1 : c.y - 1);
            n.k += ys - c.y;
            n.y = ys;
            const T fn = adv_eval<T, float>(g, n, u, nullptr, &center);
            s += (g.aypos ? -g.ay : g.ay) * g.inv_dy * fn;
        }
        grad[c.k] = s * gscale;
    }
    const int64_t bid = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const int64_t nb = (int64_t)gridDim.x * gridDim.y * gridDim.z;
    reduce_finish(acc, bid, nb, ws, lscale, loss);
}

// Mixed-precision Newton step (FP64 on all SMs): u_out = u + d, rhs =
// float(-F(u_out)), optional sum(F^2).
template <bool HAS_D, bool NORM>
__global__ void __launch_bounds__(256) adv_update_residual_kernel(
    AdvDev<double> g, const double* __restrict__ u, const float* __restrict__ d,
    double* __restrict__ uout, float* __restrict__ rhs, ReduceWs ws, double* rnorm2) {
    Cell c;
    double acc = 0.0;
    if (cell_of(g, &c)) {
        double center;
        const double f = adv_eval<double, float>(g, c, u, HAS_D ? d : nullptr, &center);
        if constexpr (HAS_D) uout[c.k] = center;
        rhs[c.k] = (float)(-f);
        if constexpr (NORM) acc = f * f;
    }
    if constexpr (NORM) {
        const int64_t bid = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        reduce_finish(acc, bid, (int64_t)gridDim.x * gridDim.y * gridDim.z, ws, 1.0, rnorm2);
    }
}

// ---------------------------------------------------------------------------
// Multigrid (FP32).  Damped Jacobi: x_out = x + omega (b - J x) / D; with
// x = NULL the iterate is zero and x_out = omega b / D.
__global__ void __launch_bounds__(256) adv_jacobi_kernel(AdvDev<float> g, const float* __restrict__ x,
                                                         const float* __restrict__ b,
                                                         float* __restrict__ xout, float omega,
                                                         float* __restrict__ r_out) {
    Cell c;
    if (!cell_of(g, &c)) return;
    const float bb = __ldg(b + c.k);
    if (!x) {
        xout[c.k] = omega * bb * g.inv_D;
        return;
    }
    float center;
    const float jx = adv_eval<float, float>(g, c, x, nullptr, &center);
    const float r = bb - jx;
    if (xout) xout[c.k] = center + omega * r * g.inv_D;
    if (r_out) r_out[c.k] = r;
}

// Cell-centred full weighting along one axis: coarse c receives fine 2c-1,
// 2c, 2c+1, 2c+2 with weights 1/8, 3/8, 3/8, 1/8 (the transpose of linear
// prolongation, halved); at a clamped end the outside weight folds onto the
// end cell.
struct W4 {
    int idx[4];
    float w[4];
};

__device__ __forceinline__ W4 fw_axis(int c, int nf, bool periodic) {
    W4 r;
    const int f0 = 2 * c - 1, f3 = 2 * c + 2;
    r.idx[0] = f0; r.w[0] = 0.125f;
    r.idx[1] = 2 * c; r.w[1] = 0.375f;
    r.idx[2] = 2 * c + 1; r.w[2] = 0.375f;
    r.idx[3] = f3; r.w[3] = 0.125f;
    if (periodic) {
        if (f0 < 0) r.idx[0] = f0 + nf;
        if (f3 >= nf) r.idx[3] = f3 - nf;
    } else {
        if (f0 < 0) { r.idx[0] = 0; }       // fine 0 keeps its 1/4 on coarse 0
        if (f3 >= nf) { r.idx[3] = nf - 1; }
    }
    return r;
}

__global__ void __launch_bounds__(256) adv_restrict_kernel(const float* __restrict__ r, int nt,
                                                           int nx, int ny, float* __restrict__ rc) {
    const int nxc = nx / 2, nyc = ny / 2;
    const int yc = blockIdx.x * blockDim.x + threadIdx.x;
    const int xc = blockIdx.y, tc = blockIdx.z;
    if (yc >= nyc) return;
    const W4 wt = fw_axis(tc, nt, false), wx = fw_axis(xc, nx, true), wy = fw_axis(yc, ny, true);
    float s = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const float* row = r + ((int64_t)wt.idx[a] * nx + wx.idx[b]) * ny;
            const float wab = wt.w[a] * wx.w[b];
#pragma unroll
            for (int c = 0; c < 4; ++c) s += wab * wy.w[c] * __ldg(row + wy.idx[c]);
        }
    }
    rc[((int64_t)tc * nxc + xc) * nyc + yc] = s;
}

// x[fine] += trilinear interpolation of the coarse correction e (t clamped,
// x and y periodic): fine 2c gets 3/4 e[c] + 1/4 e[c-1], fine 2c+1 gets
// 3/4 e[c] + 1/4 e[c+1] per axis.
__device__ __forceinline__ void lin_axis(int f, int nc, bool periodic, int* i0, int* i1,
                                         float* w0, float* w1) {
    const int c = f >> 1;
    int o = (f & 1) ? c + 1 : c - 1;
    if (periodic) {
        o = o < 0 ? o + nc : (o >= nc ? o - nc : o);
    } else {
        o = o < 0 ? 0 : (o >= nc ? nc - 1 : o);
    }
    *i0 = c;
    *i1 = o;
    *w0 = 0.75f;
    *w1 = 0.25f;
}

// One thread per coarse y index c: fine y = 2c and 2c+1 share the coarse
// values c-1, c, c+1 of the four (t, x) coarse rows, so a thread loads 12
// coarse values for two fine cells and updates them with one 8-byte access.
__global__ void __launch_bounds__(256) adv_prolong_add_kernel(const float* __restrict__ e, int nt,
                                                              int nx, int ny, float* __restrict__ x) {
    const int ntc = nt / 2, nxc = nx / 2, nyc = ny / 2;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;  // coarse y
    const int xx = blockIdx.y, t = blockIdx.z;
    if (c >= nyc) return;
    int ti[2], xi[2];
    float tw[2], xw[2];
    lin_axis(t, ntc, false, &ti[0], &ti[1], &tw[0], &tw[1]);
    lin_axis(xx, nxc, true, &xi[0], &xi[1], &xw[0], &xw[1]);
    const int cm = c == 0 ? nyc - 1 : c - 1;
    const int cp = c + 1 == nyc ? 0 : c + 1;
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const float* row = e + ((int64_t)ti[a] * nxc + xi[b]) * nyc;
            const float w = tw[a] * xw[b];
            const float ec = __ldg(row + c);
            s0 += w * (0.75f * ec + 0.25f * __ldg(row + cm));
            s1 += w * (0.75f * ec + 0.25f * __ldg(row + cp));
        }
    }
    float2* dst = reinterpret_cast<float2*>(x + ((int64_t)t * nx + xx) * ny + 2 * c);
    float2 v = *dst;
    v.x += s0;
    v.y += s1;
    *dst = v;
}

// Dense FP64 coarsest solve x = Ainv b (Ainv: the explicit inverse of the
// coarsest operator, n <= 1024), one block.
__global__ void __launch_bounds__(256) dense_apply_kernel(int n, const double* __restrict__ Ainv,
                                                          const float* __restrict__ b,
                                                          float* __restrict__ x) {
    __shared__ double sb[1024];
    for (int k = threadIdx.x; k < n; k += blockDim.x) sb[k] = (double)b[k];
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        double s = 0.0;
        const double* row = Ainv + (int64_t)r * n;
        for (int k = 0; k < n; ++k) s += row[k] * sb[k];
        x[r] = (float)s;
    }
}

// Dense matrix of the operator (rows: cells in C order), for the coarsest
// level's direct solve.
__global__ void adv_dense_kernel(AdvDev<double> g, double* __restrict__ A) {
    Cell c;
    if (!cell_of(g, &c)) return;
    const int nx = g.nx, ny = g.ny;
    const int64_t n = (int64_t)g.nt * nx * ny;
    double* row = A + c.k * n;
    for (int64_t k = 0; k < n; ++k) row[k] = 0.0;
    row[c.k] += g.D;
    if (c.i >= 1) row[c.k - (int64_t)nx * ny] += -g.inv_dt;
    const int64_t slab = c.k - (int64_t)c.x * ny - c.y;
    const int64_t rowk = c.k - c.y;
    if (g.axpos) {
        row[slab + (int64_t)(c.x == 0 ? nx - 1 : c.x - 1) * ny + c.y] += -g.ax * g.inv_dx;
    } else {
        row[slab + (int64_t)(c.x + 1 == nx ? 0 : c.x + 1) * ny + c.y] += g.ax * g.inv_dx;
    }
    if (g.aypos) {
        row[rowk + (c.y == 0 ? ny - 1 : c.y - 1)] += -g.ay * g.inv_dy;
    } else {
        row[rowk + (c.y + 1 == ny ? 0 : c.y + 1)] += g.ay * g.inv_dy;
    }
}

// ---------------------------------------------------------------------------
// FP32 fast path (ny a multiple of 4, 16-byte aligned arrays): a thread owns 4
// consecutive y cells of one (t, x) row, loads each stencil row with one
// 16-byte access, takes the upwind y-neighbour of its first (or last) cell
// from the adjacent lane by a shuffle, and only the warp's end lanes load a
// word across the lane boundary (with the periodic wrap).  Same residual
// formula and operation order as adv_f.
struct Row4 {
    int i, x, y0;  // cell (i, x, y0 .. y0+3)
    int64_t k;     // packed index of (i, x, y0)
    bool ok;
};

__device__ __forceinline__ Row4 row4_of(const AdvDev<float>& g) {
    Row4 c;
    c.y0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    c.x = blockIdx.y * blockDim.y + threadIdx.y;
    c.i = blockIdx.z;
    c.k = ((int64_t)c.i * g.nx + c.x) * g.ny + c.y0;
    c.ok = c.y0 < g.ny && c.x < g.nx;
    return c;
}

__device__ __forceinline__ float4 ld4(const float* p, int64_t k) {
    return __ldg(reinterpret_cast<const float4*>(p + k));
}

// Residuals (init: with p_init on row 0; else the linear part J v) of the 4
// cells; also returns the centre values.  All lanes must call it (shuffles).
__device__ __forceinline__ void adv_eval4(const AdvDev<float>& g, const Row4& c,
                                          const float* __restrict__ u, float (&f)[4],
                                          float4* centre) {
    const int nx = g.nx, ny = g.ny;
    const int lane = threadIdx.x & 31;
    float4 P = make_float4(0.f, 0.f, 0.f, 0.f), PT = P, PX = P;
    if (c.ok) {
        P = ld4(u, c.k);
        if (c.i == 0) {
            if (g.p_init) PT = ld4(g.p_init, (int64_t)c.x * ny + c.y0);
        } else {
            PT = ld4(u, c.k - (int64_t)nx * ny);
        }
        const int xn = g.axpos ? (c.x == 0 ? nx - 1 : c.x - 1) : (c.x + 1 == nx ? 0 : c.x + 1);
        PX = ld4(u, c.k + (int64_t)(xn - c.x) * ny);
    }
    *centre = P;
    // y-neighbour outside the thread's 4 cells.
    const int64_t rowk = c.k - c.y0;
    float yo;
    if (g.aypos) {
        yo = __shfl_up_sync(0xffffffffu, P.w, 1);
        if (c.ok && (lane == 0 || c.y0 == 0))
            yo = __ldg(u + rowk + (c.y0 == 0 ? ny - 1 : c.y0 - 1));
    } else {
        yo = __shfl_down_sync(0xffffffffu, P.x, 1);
        if (c.ok && (lane == 31 || c.y0 + 4 >= ny))
            yo = __ldg(u + rowk + (c.y0 + 4 >= ny ? 0 : c.y0 + 4));
    }
    const float p[4] = {P.x, P.y, P.z, P.w};
    const float pt[4] = {PT.x, PT.y, PT.z, PT.w};
    const float px[4] = {PX.x, PX.y, PX.z, PX.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const float ym = e == 0 ? yo : p[e - 1];
        const float yp = e == 3 ? yo : p[e + 1];
        f[e] = adv_f(g, p[e], pt[e], px[e], px[e], ym, yp);
    }
}

__global__ void __launch_bounds__(256) adv_residual4_kernel(AdvDev<float> g,
                                                            const float* __restrict__ u,
                                                            float* __restrict__ f) {
    const Row4 c = row4_of(g);
    float r[4];
    float4 centre;
    adv_eval4(g, c, u, r, &centre);
    if (c.ok) *reinterpret_cast<float4*>(f + c.k) = make_float4(r[0], r[1], r[2], r[3]);
}

// Damped Jacobi (adv_jacobi_kernel's arithmetic, same rounding) on 4 cells
// per thread.
__global__ void __launch_bounds__(256) adv_jacobi4_kernel(AdvDev<float> g,
                                                          const float* __restrict__ x,
                                                          const float* __restrict__ b,
                                                          float* __restrict__ xout, float omega,
                                                          float* __restrict__ r_out) {
    const Row4 c = row4_of(g);
    const float iD = g.inv_D;
    if (!x) {
        if (!c.ok) return;
        const float4 B = ld4(b, c.k);
        *reinterpret_cast<float4*>(xout + c.k) = make_float4(
            omega * B.x * iD, omega * B.y * iD, omega * B.z * iD, omega * B.w * iD);
        return;
    }
    float jx[4];
    float4 P;
    adv_eval4(g, c, x, jx, &P);
    if (!c.ok) return;
    const float4 B = ld4(b, c.k);
    const float r0 = B.x - jx[0], r1 = B.y - jx[1], r2 = B.z - jx[2], r3 = B.w - jx[3];
    if (xout)
        *reinterpret_cast<float4*>(xout + c.k) =
            make_float4(P.x + omega * r0 * iD, P.y + omega * r1 * iD, P.z + omega * r2 * iD,
                        P.w + omega * r3 * iD);
    if (r_out) *reinterpret_cast<float4*>(r_out + c.k) = make_float4(r0, r1, r2, r3);
}

inline bool adv_vec4(const AdvDev<float>& g, std::initializer_list<const void*> ptrs) {
    if (g.ny % 4) return false;
    for (const void* q : ptrs)
        if (q && (reinterpret_cast<uintptr_t>(q) & 15u)) return false;
    return true;
}

// Blocks of about 256 threads: whole warps along y (a warp never spans two x
// rows, so its shuffles stay in one row), then as many x rows as fit.
inline void adv_launch_dims4(int nt, int nx, int ny, dim3* grid, dim3* block) {
    const int per = ny / 4;
    const int bx = per >= 256 ? 256 : ((per + 31) / 32) * 32;
    int by = 256 / bx;
    if (by > nx) by = nx;
    *block = dim3(bx, by);
    *grid = dim3((per + bx - 1) / bx, (nx + by - 1) / by, nt);
}

template <typename T>
int residual_impl(const odil_advect_params* p, const T* u, T* f, void* stream, bool init) {
    AdvDev<T> g;
    int st = make_adv<T>(p, &g, init);
    if (st) return st;
    if (!u || !f) return ODIL_ERR_ARG;
    if constexpr (sizeof(T) == 4) {
        if (adv_vec4(g, {u, f, g.p_init})) {
            dim3 grid, block;
            adv_launch_dims4(g.nt, g.nx, g.ny, &grid, &block);
            adv_residual4_kernel<<<grid, block, 0, as_stream(stream)>>>(g, u, f);
            return launch_status();
        }
    }
    dim3 grid, block;
    adv_launch_dims(g.nt, g.nx, g.ny, &grid, &block);
    adv_residual_kernel<T><<<grid, block, 0, as_stream(stream)>>>(g, u, f);
    return launch_status();
}

template <typename T>
int jtv_impl(const odil_advect_params* p, const T* w, T* out, void* stream) {
    AdvDev<T> g;
    int st = make_adv<T>(p, &g, false);
    if (st) return st;
    if (!w || !out) return ODIL_ERR_ARG;
    dim3 grid, block;
    adv_launch_dims(g.nt, g.nx, g.ny, &grid, &block);
    adv_jtv_kernel<T><<<grid, block, 0, as_stream(stream)>>>(g, w, out);
    return launch_status();
}

inline int64_t adv_blocks(const odil_advect_params* p) {
    dim3 grid, block;
    adv_launch_dims((int)p->nt, (int)p->nx, (int)p->ny, &grid, &block);
    return (int64_t)grid.x * grid.y * grid.z;
}

template <typename T>
int loss_grad_impl(const odil_advect_params* p, const T* u, T* grad, double* loss, void* ws,
                   int64_t ws_bytes, void* stream) {
    AdvDev<T> g;
    int st = make_adv<T>(p, &g, true);
    if (st) return st;
    if (!u || !grad || !loss) return ODIL_ERR_ARG;
    if (!ws || ws_bytes < reduce_ws_bytes(adv_blocks(p))) return ODIL_ERR_WORKSPACE;
    dim3 grid, block;
    adv_launch_dims(g.nt, g.nx, g.ny, &grid, &block);
    const double n = (double)g.nt * g.nx * g.ny;
    adv_loss_grad_kernel<T><<<grid, block, 0, as_stream(stream)>>>(
        g, u, grad, reduce_ws(ws), loss, (T)(2.0 / n), 1.0 / n);
    return launch_status();
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int64_t odil_advect_workspace_bytes(const odil_advect_params* p) {
    if (!p || p->nt < 1 || p->nx < 1 || p->ny < 1) return 0;
    return reduce_ws_bytes(adv_blocks(p));
}
ODIL_API int odil_advect_residual_f32(const odil_advect_params* p, const float* u, float* f,
                                      void* stream) {
    return residual_impl<float>(p, u, f, stream, true);
}
ODIL_API int odil_advect_residual_f64(const odil_advect_params* p, const double* u, double* f,
                                      void* stream) {
    return residual_impl<double>(p, u, f, stream, true);
}
ODIL_API int odil_advect_jv_f32(const odil_advect_params* p, const float* v, float* out,
                                void* stream) {
    return residual_impl<float>(p, v, out, stream, false);
}
ODIL_API int odil_advect_jv_f64(const odil_advect_params* p, const double* v, double* out,
                                void* stream) {
    return residual_impl<double>(p, v, out, stream, false);
}
ODIL_API int odil_advect_jtv_f32(const odil_advect_params* p, const float* w, float* out,
                                 void* stream) {
    return jtv_impl<float>(p, w, out, stream);
}
ODIL_API int odil_advect_jtv_f64(const odil_advect_params* p, const double* w, double* out,
                                 void* stream) {
    return jtv_impl<double>(p, w, out, stream);
}
ODIL_API int odil_advect_loss_grad_f32(const odil_advect_params* p, const float* u, float* grad,
                                       double* loss, void* workspace, int64_t workspace_bytes,
                                       void* stream) {
    return loss_grad_impl<float>(p, u, grad, loss, workspace, workspace_bytes, stream);
}
ODIL_API int odil_advect_loss_grad_f64(const odil_advect_params* p, const double* u, double* grad,
                                       double* loss, void* workspace, int64_t workspace_bytes,
                                       void* stream) {
    return loss_grad_impl<double>(p, u, grad, loss, workspace, workspace_bytes, stream);
}
ODIL_API int odil_advect_update_residual_mixed(const odil_advect_params* p, const double* u,
                                               const float* d, double* u_out, float* rhs,
                                               double* rnorm2, void* workspace,
                                               int64_t workspace_bytes, void* stream) {
    AdvDev<double> g;
    int st = make_adv<double>(p, &g, true);
    if (st) return st;
    if (!u || !rhs || (d && !u_out) || (d && u_out == u)) return ODIL_ERR_ARG;
    ReduceWs ws = {};
    if (rnorm2) {
        if (!workspace || workspace_bytes < reduce_ws_bytes(adv_blocks(p)))
            return ODIL_ERR_WORKSPACE;
        ws = reduce_ws(workspace);
    }
    dim3 grid, block;
    adv_launch_dims(g.nt, g.nx, g.ny, &grid, &block);
    cudaStream_t s = as_stream(stream);
    if (d) {
        if (rnorm2)
            adv_update_residual_kernel<true, true><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
        else
            adv_update_residual_kernel<true, false><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
    } else {
        if (rnorm2)
            adv_update_residual_kernel<false, true><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
        else
            adv_update_residual_kernel<false, false><<<grid, block, 0, s>>>(g, u, d, u_out, rhs, ws, rnorm2);
    }
    return launch_status();
}
ODIL_API int odil_advect_mg_jacobi(const odil_advect_params* p, const float* x, const float* b,
                                   float* x_out, float omega, float* r_out, void* stream) {
    AdvDev<float> g;
    int st = make_adv<float>(p, &g, false);
    if (st) return st;
    if (!b || (!x_out && !r_out) || (x && x == x_out) || (!x && r_out)) return ODIL_ERR_ARG;
    dim3 grid, block;
    if (adv_vec4(g, {x, b, x_out, r_out})) {
        adv_launch_dims4(g.nt, g.nx, g.ny, &grid, &block);
        adv_jacobi4_kernel<<<grid, block, 0, as_stream(stream)>>>(g, x, b, x_out, omega, r_out);
        return launch_status();
    }
    adv_launch_dims(g.nt, g.nx, g.ny, &grid, &block);
    adv_jacobi_kernel<<<grid, block, 0, as_stream(stream)>>>(g, x, b, x_out, omega, r_out);
    return launch_status();
}
ODIL_API int odil_advect_mg_restrict(int64_t nt, int64_t nx, int64_t ny, const float* r,
                                     float* rc, void* stream) {
    if (nt < 2 || nx < 2 || ny < 2 || nt % 2 || nx % 2 || ny % 2 || nt > 65535 || nx > 65535)
        return ODIL_ERR_SHAPE;
    if (!r || !rc) return ODIL_ERR_ARG;
    dim3 grid, block;
    adv_launch_dims((int)nt / 2, (int)nx / 2, (int)ny / 2, &grid, &block);
    adv_restrict_kernel<<<grid, block, 0, as_stream(stream)>>>(r, (int)nt, (int)nx, (int)ny, rc);
    return launch_status();
}
ODIL_API int odil_advect_mg_prolong_add(int64_t nt, int64_t nx, int64_t ny, const float* e,
                                        float* x, void* stream) {
    if (nt < 2 || nx < 2 || ny < 2 || nt % 2 || nx % 2 || ny % 2 || nt > 65535 || nx > 65535)
        return ODIL_ERR_SHAPE;
    if (!e || !x) return ODIL_ERR_ARG;
    dim3 grid, block;
    adv_launch_dims((int)nt, (int)nx, (int)ny / 2, &grid, &block);  // coarse y per thread
    adv_prolong_add_kernel<<<grid, block, 0, as_stream(stream)>>>(e, (int)nt, (int)nx, (int)ny, x);
    return launch_status();
}
ODIL_API int odil_advect_dense(const odil_advect_params* p, double* A, void* stream) {
    AdvDev<double> g;
    int st = make_adv<double>(p, &g, false);
    if (st) return st;
    if (p->nt * p->nx * p->ny > 1024) return ODIL_ERR_SHAPE;
    if (!A) return ODIL_ERR_ARG;
    dim3 grid, block;
    adv_launch_dims(g.nt, g.nx, g.ny, &grid, &block);
    adv_dense_kernel<<<grid, block, 0, as_stream(stream)>>>(g, A);
    return launch_status();
}
ODIL_API int odil_dense_apply_f64(int64_t n, const double* Ainv, const float* b, float* x,
                                  void* stream) {
    if (n < 1 || n > 1024) return ODIL_ERR_SHAPE;
    if (!Ainv || !b || !x) return ODIL_ERR_ARG;
    dense_apply_kernel<<<1, 256, 0, as_stream(stream)>>>((int)n, Ainv, b, x);
    return launch_status();
}
