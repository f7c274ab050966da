// Device-side pieces of the 1D wave operator shared by the single-instance
// (wave.cu) and batched (batch.cu) kernels: parameters, the residual of one
// cell, the Jacobian's column-class factors, the J^T gather, and the
// forward-substitution march.  See wave.cu for the operator and its
// reference (wave.py:67-122).
#pragma once

#include <type_traits>

#include "common.cuh"

namespace odil {
namespace wavedev {


template <typename T>
struct WaveDev {
    int nt, nx;
    T inv_dt, inv_dx2, c2, half_dt;
    T A, B;       // 1/dt^2, c^2/dx^2
    T dt2, lam2;  // dt^2, c^2 dt^2 / dx^2
    const T* init_u;
    const T* init_ut;
    const T* left_u;
    const T* right_u;
};

template <typename T>
int make_dev(const odil_wave_params* p, WaveDev<T>* g, bool with_bc) {
    if (!p) return ODIL_ERR_ARG;
    if (p->nt < 1 || p->nx < 1 || p->nt > (1 << 30) || p->nx > (1 << 30) ||
        p->nt * p->nx > (int64_t(1) << 31) - 1)
        return ODIL_ERR_SHAPE;
    if (!(p->dt > 0) || !(p->dx > 0)) return ODIL_ERR_ARG;
    g->nt = (int)p->nt;
    g->nx = (int)p->nx;
    const double inv_dt = 1.0 / p->dt;
    const double inv_dx2 = 1.0 / (p->dx * p->dx);
    g->inv_dt = (T)inv_dt;
    g->inv_dx2 = (T)inv_dx2;
    g->c2 = (T)(p->c * p->c);
    g->half_dt = (T)(0.5 * p->dt);
    g->A = (T)(inv_dt * inv_dt);
    g->B = (T)(p->c * p->c * inv_dx2);
    g->dt2 = (T)(p->dt * p->dt);
    g->lam2 = (T)(p->c * p->c * p->dt * p->dt * inv_dx2);
    g->init_u = with_bc ? (const T*)p->init_u : nullptr;
    g->init_ut = with_bc ? (const T*)p->init_ut : nullptr;
    g->left_u = with_bc ? (const T*)p->left_u : nullptr;
    g->right_u = with_bc ? (const T*)p->right_u : nullptr;
    return ODIL_OK;
}

template <typename T>
__device__ __forceinline__ T opt_ld(const T* p, int k) {
    return p ? __ldg(p + k) : T(0);
}

// Residual of cell (i, j) from its five stencil values, in the operation order
// of wave.py:106-118.  The boundary data come from the callables init_u(j),
// init_ut(j), left(i-1), right(i-1) (called only where they enter).
template <typename T, typename IU, typename IUT, typename LB, typename RB>
__device__ __forceinline__ T wave_f_with(const WaveDev<T>& g, int i, int j, T u, T utm, T utmm,
                                         T uxm, T uxp, IU init_u, IUT init_ut, LB left,
                                         RB right) {
    if (i == 0) {
        return u - (init_u(j) + g.half_dt * init_ut(j));
    }
    if (j == 0) uxm = (uxp - T(6) * utm + T(8) * left(i - 1)) / T(3);
    if (j == g.nx - 1) uxp = (uxm - T(6) * utm + T(8) * right(i - 1)) / T(3);
    const T u_t_tm = (u - utm) * g.inv_dt;
    const T u_t_tmm = (i == 1) ? init_ut(j) : (utm - utmm) * g.inv_dt;
    const T u_tt = (u_t_tm - u_t_tmm) * g.inv_dt;
    const T u_xx = (uxm - T(2) * utm + uxp) * g.inv_dx2;
    return u_tt - g.c2 * u_xx;
}

// wave_f_with reading the boundary data from global memory.
template <typename T>
__device__ __forceinline__ T wave_f(const WaveDev<T>& g, int i, int j, T u, T utm, T utmm,
                                    T uxm, T uxp) {
    return wave_f_with(
        g, i, j, u, utm, utmm, uxm, uxp, [&](int k) { return opt_ld(g.init_u, k); },
        [&](int k) { return opt_ld(g.init_ut, k); }, [&](int k) { return opt_ld(g.left_u, k); },
        [&](int k) { return opt_ld(g.right_u, k); });
}

// Column-class factors of d(u_xx_raw)/d(slot) (see the header comment).
template <typename T>
__device__ __forceinline__ T k_tm(int col, int nx) {
    if (nx == 1) return T(20.0 / 3.0);
    return (col == 0 || col == nx - 1) ? T(4) : T(2);
}
template <typename T>
__device__ __forceinline__ T k_xm(int col, int nx) {
    if (nx == 1 || col == 0) return T(0);
    return col == nx - 1 ? T(4.0 / 3.0) : T(1);
}
template <typename T>
__device__ __forceinline__ T k_xp(int col, int nx) {
    if (nx == 1) return T(4.0 / 9.0);
    if (col == nx - 1) return T(0);
    return col == 0 ? T(4.0 / 3.0) : T(1);
}

// Gather of J^T at cell (a, b): sum over the rows that read u[a, b].
// f_* are the values of the multiplied vector at the dependent rows.
template <typename T>
__device__ __forceinline__ T wave_gather(const WaveDev<T>& g, int a, int b, T f_u, T f_tm,
                                         T f_tmm, T f_xm, T f_xp) {
    const int nt = g.nt, nx = g.nx;
    T s = (a == 0 ? T(1) : g.A) * f_u;
    if (a + 1 < nt) {
        const T ctm = (a + 1 == 1 ? -g.A : T(-2) * g.A) + g.B * k_tm<T>(b, nx);
        s += ctm * f_tm;
        const int bp = (b + 1 == nx) ? 0 : b + 1;
        const int bm = (b == 0) ? nx - 1 : b - 1;
        s -= g.B * (k_xm<T>(bp, nx) * f_xm + k_xp<T>(bm, nx) * f_xp);
    }
    if (a + 2 < nt) s += g.A * f_tmm;
    return s;
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
// lg_strip runs the strips of tile (bx, by) (column group bx of LG_WARPS
// strips, rows [TY by, TY by + TY)) and returns the thread's share of the
// sum of f^2 over the tile's output rows; the single-instance kernel and the
// batched one (batch.cu) call it.
constexpr int LG_WARPS = 4;
constexpr int LG_OUT = 30;  // output columns per warp

template <typename T, int TY>
__device__ __forceinline__ T lg_strip(const WaveDev<T>& g, const T* __restrict__ u,
                                      T* __restrict__ grad, int bx, int by, T gscale) {
    const int nt = g.nt, nx = g.nx;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int c0 = (bx * LG_WARPS + warp) * LG_OUT;  // first output column
    const int a0 = by * TY;
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
    return lsum;
}

// ---------------------------------------------------------------------------
// Accurate residual of a field held as an unevaluated sum of two FP32 arrays,
// hi + lo, without FP64 arithmetic at interior cells.  In the interior (i >= 2,
// 0 < j < nx-1) the residual of wave_f equals
//   F = A (u0 + u2) + C u1 - B (um + up),  C = 2B - 2A,
// (u0, u1, u2 = rows i, i-1, i-2 at column j; um, up = row i-1 at j -+ 1).
// Each coefficient is split into FP32 hi + lo parts; every product of a hi
// coefficient with a hi value is formed exactly (p + e, e by FMA) and the p are
// summed with Knuth's two-sum, so the only roundings are those of the small
// correction terms: the result carries about 2^-48 of the largest term, the
// accuracy a mixed-precision Newton step needs of its right-hand side (GB300's
// FP64 pipe, ~1/64 of FP32, would otherwise bound the step).  Boundary cells
// (rows 0, 1 and columns 0, nx-1) use wave_f in FP64.
struct PairCoef {
    float ah, al, ch, cl, bh, bl;  // A, C, -B as hi + lo
};

inline void split_f64(double x, float* hi, float* lo) {
    *hi = (float)x;
    *lo = (float)(x - (double)*hi);
}

inline PairCoef pair_coef(double A, double B) {
    PairCoef k;
    split_f64(A, &k.ah, &k.al);
    split_f64(2.0 * B - 2.0 * A, &k.ch, &k.cl);
    split_f64(-B, &k.bh, &k.bl);
    return k;
}

__device__ __forceinline__ PairCoef pair_coef_dev(double A, double B) {
    PairCoef k;
    const double C = 2.0 * B - 2.0 * A;
    k.ah = __double2float_rn(A);
    k.al = __double2float_rn(A - (double)k.ah);
    k.ch = __double2float_rn(C);
    k.cl = __double2float_rn(C - (double)k.ch);
    k.bh = __double2float_rn(-B);
    k.bl = __double2float_rn(-B - (double)k.bh);
    return k;
}

// Rounding error of s = fl(a + b) (Knuth's two-sum): a + b = s + err
// exactly.  Explicit _rn intrinsics keep the compiler from contracting it.
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Load of an iterate value: read-only path (NC, the iterate is another
// kernel's output) or through L2 (the iterate was written earlier in the
// same kernel, possibly by another SM).
template <bool NC>
__device__ __forceinline__ float ld_iter(const float* p) {
    if constexpr (NC) {
        return __ldg(p);
    } else {
        return __ldcg(p);
    }
}

// -F(hi + lo) at an interior cell from its five stencil values (v: hi,
// w: lo; rows i (0), i-2 (2), i-1 (1) at column j, row i-1 at j -+ 1),
// F = A (u0 + u2) + C u1 - B (um + up) with A, C, -B as float pairs.  The
// two sums sharing a coefficient are formed exactly (value + two-sum
// error), the three hi-coefficient products exactly (product + FMA
// error), and the products summed by two-sums; every rounding error and
// the first-order small terms (lo coefficients, the sums' errors, w) go
// into one compensation c.  Error ~2^-46 of the largest term.
__device__ __forceinline__ float pair_rhs_vals(const PairCoef& k, float v0, float v2, float v1,
                                               float vm, float vp, float w0, float w2, float w1,
                                               float wm, float wp) {
    const float a = __fadd_rn(v0, v2), ea = two_sum_err(v0, v2, a);
    const float b = __fadd_rn(vm, vp), eb = two_sum_err(vm, vp, b);
    const float p1 = __fmul_rn(k.ah, a), e1 = __fmaf_rn(k.ah, a, -p1);
    const float p2 = __fmul_rn(k.ch, v1), e2 = __fmaf_rn(k.ch, v1, -p2);
    const float p3 = __fmul_rn(k.bh, b), e3 = __fmaf_rn(k.bh, b, -p3);
    const float s = __fadd_rn(p1, p2), es = two_sum_err(p1, p2, s);
    const float t = __fadd_rn(s, p3), et = two_sum_err(s, p3, t);
    float c = __fadd_rn(__fadd_rn(__fadd_rn(es, et), __fadd_rn(e1, e2)), e3);
    c = __fmaf_rn(k.al, a, c);
    c = __fmaf_rn(k.cl, v1, c);
    c = __fmaf_rn(k.bl, b, c);
    c = __fmaf_rn(k.ah, ea, c);
    c = __fmaf_rn(k.bh, eb, c);
    c = __fmaf_rn(k.ah, __fadd_rn(w0, w2), c);
    c = __fmaf_rn(k.ch, w1, c);
    c = __fmaf_rn(k.bh, __fadd_rn(wm, wp), c);
    return -__fadd_rn(t, c);
}

// -F(hi + lo) at interior cell (i, j) rounded to FP32.  lo may be null.
template <bool NC = true>
__device__ __forceinline__ float pair_interior_rhs(const PairCoef& k, const float* __restrict__ hi,
                                                   const float* __restrict__ lo, int64_t c0,
                                                   int nx) {
    const int64_t c1 = c0 - nx, c2 = c0 - 2 * (int64_t)nx;
    const float v0 = ld_iter<NC>(hi + c0), v2 = ld_iter<NC>(hi + c2), v1 = ld_iter<NC>(hi + c1);
    const float vm = ld_iter<NC>(hi + c1 - 1), vp = ld_iter<NC>(hi + c1 + 1);
    float w0 = 0.f, w2 = 0.f, w1 = 0.f, wm = 0.f, wp = 0.f;
    if (lo) {
        w0 = ld_iter<NC>(lo + c0);
        w2 = ld_iter<NC>(lo + c2);
        w1 = ld_iter<NC>(lo + c1);
        wm = ld_iter<NC>(lo + c1 - 1);
        wp = ld_iter<NC>(lo + c1 + 1);
    }
    return pair_rhs_vals(k, v0, v2, v1, vm, vp, w0, w2, w1, wm, wp);
}

// -F(hi + lo) at any cell: the float-pair form inside, FP64 wave_f on the
// boundary rows and columns.
template <bool NC = true>
__device__ __forceinline__ float pair_cell_rhs(const WaveDev<double>& g, const PairCoef& k,
                                               const float* __restrict__ hi,
                                               const float* __restrict__ lo, int i, int j) {
    const int nx = g.nx;
    const int64_t c0 = (int64_t)i * nx + j;
    if (i >= 2 && j >= 1 && j + 1 < nx) return pair_interior_rhs<NC>(k, hi, lo, c0, nx);
    auto val = [&](int ii, int jj) -> double {
        const int64_t kk = (int64_t)ii * nx + jj;
        double v = (double)ld_iter<NC>(hi + kk);
        if (lo) v += (double)ld_iter<NC>(lo + kk);
        return v;
    };
    const double uc = val(i, j);
    double utm = 0, utmm = 0, uxm = 0, uxp = 0;
    if (i >= 1) {
        utm = val(i - 1, j);
        uxm = val(i - 1, j == 0 ? nx - 1 : j - 1);
        uxp = val(i - 1, j + 1 == nx ? 0 : j + 1);
    }
    if (i >= 2) utmm = val(i - 2, j);
    return (float)(-wave_f(g, i, j, uc, utm, utmm, uxm, uxp));
}

// -F(hi + lo) (KIND 1) or -F(0) (KIND 0) at a boundary cell (row 0 or 1,
// column 0 or nx-1) in FP64.
template <int KIND, bool NC = true>
__device__ __forceinline__ float bnd_cell_rhs(const WaveDev<double>& g, const PairCoef& k,
                                              const float* __restrict__ hi,
                                              const float* __restrict__ lo, int i, int j) {
    if (KIND == 0) return (float)(-wave_f(g, i, j, 0.0, 0.0, 0.0, 0.0, 0.0));
    return pair_cell_rhs<NC>(g, k, hi, lo, i, j);
}

// Boundary cells of an nt x nx grid: rows 0 and 1 (all columns), then columns
// 0 and nx-1 of rows 2.. .  Count and the cell of index t.
__host__ __device__ __forceinline__ int64_t bnd_count(int nt, int nx) {
    const int r = nt < 2 ? nt : 2;
    const int c = nx < 2 ? nx : 2;
    return (int64_t)r * nx + (int64_t)(nt > 2 ? nt - 2 : 0) * c;
}
__device__ __forceinline__ void bnd_cell(int64_t t, int nt, int nx, int* i, int* j) {
    const int r = nt < 2 ? nt : 2;
    const int64_t head = (int64_t)r * nx;
    if (t < head) {
        *i = (int)(t / nx);
        *j = (int)(t - (int64_t)*i * nx);
    } else {
        const int c = nx < 2 ? nx : 2;
        const int64_t u = t - head;
        *i = 2 + (int)(u / c);
        *j = (u % c) == 0 ? 0 : nx - 1;
    }
}

// ---------------------------------------------------------------------------
// Forward substitution J x = b, one block marching the rows (the rows are a
// dependency chain; the parallelism is across x).  Thread t owns the CPT
// contiguous columns [CPT t, CPT t + CPT); rows i-1 and i-2 of its columns stay
// in registers.  The x-neighbours of row i-1 at the ends of a thread's run come
// from the adjacent lanes by warp shuffles; only the two end values of each
// warp go through shared memory (a two-row-parity buffer), so one
// __syncthreads per row orders them and the shared-memory pipe carries a few
// words per warp and row.  Right-hand-side rows stream into a PF-row
// shared-memory ring with cp.async (one CPT-wide copy per thread and row, PF-1
// rows ahead of the march), so the HBM latency is off the dependency chain;
// each thread copies and later reads only its own columns, so
// cp.async.wait_group alone orders the ring.  The row loop is unrolled by PF so
// ring slots are compile-time constants.  No FP64 arithmetic in the FP32
// instance: GB300's FP64 pipe would bound the chain.
//
// At the two ends of a row the periodic neighbour (column nx-1 left of column
// 0, column 0 right of column nx-1) has coefficient zero (k_xm(0) = k_xp(nx-1)
// = 0), so the march uses 0 there; for nx = 1 the right neighbour is the cell
// itself, with k_xp = 4/9.
constexpr int kMarchMaxWarps = 32;

__device__ __forceinline__ void cp_async_n(void* smem, const void* gmem, int bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (bytes == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
    } else if (bytes == 8) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

template <typename T, int CPT>
struct Chunk {
    T v[CPT];
};

// VEC: the thread's CPT columns are contiguous and 16/8/4-byte aligned in
// global memory (nx % CPT == 0 and aligned pointers), so the ring copy and the
// solution store are single vector accesses.
// REG: the right-hand-side rows are prefetched into registers (PF rows of
// the thread's CPT values, loads in flight until first use) instead of the
// shared-memory ring, which takes the ring's write and read off the L1 pipe
// and its read off the row-to-row dependency chain; the shared memory then
// holds only the edge words.
template <typename T, int CPT>
__device__ __forceinline__ void ld_run(T (&out)[CPT], const T* __restrict__ p) {
    constexpr int bytes = CPT * (int)sizeof(T);
    if constexpr (bytes % 16 == 0) {
#pragma unroll
        for (int o = 0; o < bytes / 16; ++o) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(p) + o);
            memcpy(reinterpret_cast<char*>(out) + 16 * o, &v, 16);
        }
    } else if constexpr (bytes == 8) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        memcpy(out, &v, 8);
    } else {
#pragma unroll
        for (int c = 0; c < CPT; ++c) out[c] = __ldg(p + c);
    }
}

template <typename T, int CPT, int PF, bool VEC, bool REG = false>
__device__ __forceinline__ void march_instance(const WaveDev<T>& g, const T* __restrict__ b,
                                               T* __restrict__ x, unsigned char* smem_raw) {
    static_assert(PF % 2 == 0, "row parity follows the ring slot");
    const int nx = g.nx, nt = g.nt;
    T* ring = reinterpret_cast<T*>(smem_raw);  // [PF][nx] right-hand sides (ring mode)
    T* edge = REG ? ring : ring + PF * nx;     // [2 parity][2 end][kMarchMaxWarps]
    T pre[REG ? PF : 1][CPT];                  // register ring (REG mode)
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarp = (blockDim.x + 31) >> 5;
    const int j0 = threadIdx.x * CPT;
    const bool active = j0 < nx;
    T kxm[CPT], ktm[CPT], kxp[CPT], d1[CPT], d2[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
        const int j = j0 + c;
        const int jj = j < nx ? j : 0;
        ktm[c] = k_tm<T>(jj, nx);
        kxm[c] = k_xm<T>(jj, nx);
        kxp[c] = k_xp<T>(jj, nx);
        d1[c] = T(0);
        d2[c] = T(0);
    }
    // Edge slots this thread reads (every lane of a warp reads the same word,
    // a broadcast) and whether the value there is a real neighbour.
    // The first warp's left word and the last warp's right word are the
    // warp's own ends: finite values that meet k_xm(0) = 0 / k_xp(nx-1) = 0.
    const int wl = warp > 0 ? warp - 1 : 0;
    const int wr = warp + 1 < nwarp ? warp + 1 : warp;
    const bool use_l = lane == 0, use_r = lane == 31;
    const bool self_r = nx == 1;
    // Every thread's run lies inside the row (no columns past its end).
    const bool full = (int64_t)nwarp * 32 * CPT == nx;
    // Both parities start at 0: row 0 scales its neighbours by 0, which must
    // not meet a stale non-finite word.
    for (int e = threadIdx.x; e < 4 * kMarchMaxWarps; e += blockDim.x) edge[e] = T(0);
    __syncthreads();
    const T* src = b + j0;  // next right-hand-side row to prefetch
    T* dst = x + j0;        // solution row being written
    auto issue = [&](int row, int slot) {
        if constexpr (REG) {
            if (active && row < nt) {
                if constexpr (VEC) {
                    ld_run<T, CPT>(pre[slot], src);
                } else {
#pragma unroll
                    for (int c = 0; c < CPT; ++c)
                        pre[slot][c] = j0 + c < nx ? __ldg(src + c) : T(0);
                }
            }
            src += nx;
            return;
        }
        if (active && row < nt) {
            T* to = ring + slot * nx + j0;
            if constexpr (VEC) {
                constexpr int bytes = CPT * (int)sizeof(T);
                if constexpr (bytes <= 16) {
                    cp_async_n(to, src, bytes);
                } else {
#pragma unroll
                    for (int off = 0; off < bytes; off += 16)
                        cp_async_n(reinterpret_cast<char*>(to) + off,
                                   reinterpret_cast<const char*>(src) + off, 16);
                }
            } else {
#pragma unroll
                for (int c = 0; c < CPT; ++c)
                    if (j0 + c < nx) cp_async_n(to + c, src + c, (int)sizeof(T));
            }
        }
        src += nx;
        cp_async_commit();
    };
#pragma unroll
    for (int s = 0; s < PF - 1; ++s) issue(s, s);
    // One row; GEN: the general step (rows 0 and 1 of J, rows past nt,
    // threads past the row end); the middle blocks of PF rows, where none of
    // these can occur, use the check-free step.
    auto row = [&](auto gen_tag, int i, int s) {
        constexpr bool GEN = decltype(gen_tag)::value;
        issue(i + PF - 1, (s + PF - 1) % PF);
        // Row 0 of J is the identity; row 1 has no u[i-2] term.
        const T c_rhs = GEN ? (i == 0 ? T(1) : g.dt2) : g.dt2;
        const T c_d1 = GEN ? (i == 1 ? T(1) : T(2)) : T(2);
        const T c_lam = GEN ? (i == 0 ? T(0) : g.lam2) : g.lam2;
        // x-neighbours of row i-1 at the ends of this thread's run.
        const T* eprv = edge + ((s & 1) ^ 1) * 2 * kMarchMaxWarps;  // PF is even
        const T el = eprv[kMarchMaxWarps + wl];
        const T er = eprv[wr];
        const T sl = __shfl_up_sync(0xffffffffu, d1[CPT - 1], 1);
        const T sr = __shfl_down_sync(0xffffffffu, d1[0], 1);
        const T left = use_l ? el : sl;
        const T right = self_r ? d1[0] : (use_r ? er : sr);
        // Threads past the row end read nothing (their columns lie outside
        // the ring) and carry zeros.
        Chunk<T, CPT> rhs;
        if constexpr (REG) {
#pragma unroll
            for (int c = 0; c < CPT; ++c) rhs.v[c] = (!GEN || active) ? pre[s][c] : T(0);
        } else if constexpr (VEC) {
            cp_async_wait<PF - 1>();  // this thread's copy of row i has landed
            const T* rrow = ring + s * nx + j0;
            if (!GEN || active) {
                rhs = *reinterpret_cast<const Chunk<T, CPT>*>(rrow);
            } else {
#pragma unroll
                for (int c = 0; c < CPT; ++c) rhs.v[c] = T(0);
            }
        } else {
            cp_async_wait<PF - 1>();
            const T* rrow = ring + s * nx + j0;
#pragma unroll
            for (int c = 0; c < CPT; ++c) rhs.v[c] = j0 + c < nx ? rrow[c] : T(0);
        }
        Chunk<T, CPT> out;
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const T xm = c == 0 ? left : d1[c - 1];
            const T xp = c == CPT - 1 ? right : d1[c + 1];
            const T tprev = c_d1 * d1[c] - d2[c];
            out.v[c] = c_rhs * rhs.v[c] + tprev +
                       c_lam * (kxm[c] * xm - ktm[c] * d1[c] + kxp[c] * xp);
        }
        if (!GEN || active) {
            if constexpr (VEC) {
                *reinterpret_cast<Chunk<T, CPT>*>(dst) = out;
            } else {
#pragma unroll
                for (int c = 0; c < CPT; ++c) {
                    if (j0 + c < nx) dst[c] = out.v[c];
                }
            }
        }
        if (GEN || !VEC) {
#pragma unroll
            for (int c = 0; c < CPT; ++c)
                if (j0 + c >= nx) out.v[c] = T(0);  // columns past the row end
        }
        dst += nx;
        T* ecur = edge + (s & 1) * 2 * kMarchMaxWarps;
        if (use_l) ecur[warp] = out.v[0];
        if (use_r) ecur[kMarchMaxWarps + warp] = out.v[CPT - 1];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            d2[c] = d1[c];
            d1[c] = out.v[c];
        }
        __syncthreads();
    };
    for (int i0 = 0; i0 < nt; i0 += PF) {
        if (i0 == 0 || i0 + PF > nt || !full) {
#pragma unroll
            for (int s = 0; s < PF; ++s) {
                if (i0 + s >= nt) break;
                row(std::true_type{}, i0 + s, s);
            }
        } else {
#pragma unroll
            for (int s = 0; s < PF; ++s) row(std::false_type{}, i0 + s, s);
        }
    }
    if constexpr (!REG) cp_async_wait<0>();
}

// Largest block of a march with CPT columns per thread and PF prefetched
// rows: the register ring of the FP32 march needs CPT PF registers on top of
// the rest; the shared-memory ring of the FP64 march needs none, but runs of
// 32 bytes or more need more than the 64 registers a 1024-thread block leaves.
template <typename T>
__host__ __device__ constexpr bool march_reg() { return sizeof(T) == 4; }

template <typename T, int CPT, int PF>
__host__ __device__ constexpr int march_max_threads() {
    return march_reg<T>() ? (CPT * PF * (int)sizeof(T) <= 64
                                 ? 1024
                                 : (CPT * PF * (int)sizeof(T) <= 128 ? 512 : 256))
                          : (CPT * sizeof(T) >= 32 ? 512 : 1024);
}

// Shared memory of a march with the ring (REG false) / of wave_march_kernel.
template <typename T>
inline size_t march_ring_smem_bytes(int nx, int pf) {
    return (size_t)pf * nx * sizeof(T) + 4 * kMarchMaxWarps * sizeof(T);
}

template <typename T>
inline size_t march_smem_bytes(int nx, int pf) {
    return march_reg<T>() ? 4 * kMarchMaxWarps * sizeof(T) : march_ring_smem_bytes<T>(nx, pf);
}

template <typename T, int CPT, int PF, bool VEC>
__global__ void __launch_bounds__(march_max_threads<T, CPT, PF>()) wave_march_kernel(
    WaveDev<T> g, const T* __restrict__ b, T* __restrict__ x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    march_instance<T, CPT, PF, VEC, march_reg<T>()>(g, b, x, smem_raw);
}


}  // namespace wavedev
}  // namespace odil
