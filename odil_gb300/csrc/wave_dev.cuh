// Device-side pieces of the 1D wave operator shared by the single-instance
// (wave.cu) and batched (batch.cu) kernels: parameters, the residual of one
// cell, the Jacobian's column-class factors, the J^T gather, and the
// forward-substitution march.  See wave.cu for the operator and its
// reference (wave.py:67-122).
#pragma once

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
// of wave.py:106-118.
template <typename T>
__device__ __forceinline__ T wave_f(const WaveDev<T>& g, int i, int j, T u, T utm, T utmm,
                                    T uxm, T uxp) {
    if (i == 0) {
        return u - (opt_ld(g.init_u, j) + g.half_dt * opt_ld(g.init_ut, j));
    }
    if (j == 0) uxm = (uxp - T(6) * utm + T(8) * opt_ld(g.left_u, i - 1)) / T(3);
    if (j == g.nx - 1) uxp = (uxm - T(6) * utm + T(8) * opt_ld(g.right_u, i - 1)) / T(3);
    const T u_t_tm = (u - utm) * g.inv_dt;
    const T u_t_tmm = (i == 1) ? opt_ld(g.init_ut, j) : (utm - utmm) * g.inv_dt;
    const T u_tt = (u_t_tm - u_t_tmm) * g.inv_dt;
    const T u_xx = (uxm - T(2) * utm + uxp) * g.inv_dx2;
    return u_tt - g.c2 * u_xx;
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
// Forward substitution J x = b, one block marching the rows (the rows are a
// dependency chain; the parallelism is across x).  Thread t owns the CPT
// contiguous columns [CPT t, CPT t + CPT).  Row i-1 lives in a double buffer in
// shared memory for the x-neighbours at the ends of a thread's run; rows i-1
// and i-2 of the own columns stay in registers.  Right-hand-side rows stream
// into a PF-row shared-memory ring with cp.async (one CPT-wide copy per thread
// and row, PF-1 rows ahead of the march), so the HBM latency is off the
// dependency chain.  Each thread copies and later reads only its own columns,
// so cp.async.wait_group alone orders the ring; one __syncthreads per row
// publishes the new row to the neighbours.  The row loop is unrolled by PF so
// ring slots are compile-time constants.  No FP64 arithmetic in the FP32
// instance: GB300's FP64 pipe would bound the chain.
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
template <typename T, int CPT, int PF, bool VEC>
__device__ __forceinline__ void march_instance(const WaveDev<T>& g, const T* __restrict__ b,
                                               T* __restrict__ x, unsigned char* smem_raw) {
    const int nx = g.nx, nt = g.nt;
    T* buf = reinterpret_cast<T*>(smem_raw);  // [2][nx] rows i-1 / i
    T* ring = buf + 2 * nx;                   // [PF][nx] right-hand sides
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
    const int jl = j0 == 0 ? nx - 1 : j0 - 1;       // left neighbour of the run
    const int jr = j0 + CPT >= nx ? (j0 + CPT) % nx : j0 + CPT;  // right neighbour
    auto issue = [&](int row, int slot) {
        if (active && row < nt) {
            const T* src = b + (int64_t)row * nx + j0;
            T* dst = ring + slot * nx + j0;
            if constexpr (VEC) {
                constexpr int bytes = CPT * (int)sizeof(T);
                if constexpr (bytes <= 16) {
                    cp_async_n(dst, src, bytes);
                } else {
#pragma unroll
                    for (int off = 0; off < bytes; off += 16)
                        cp_async_n(reinterpret_cast<char*>(dst) + off,
                                   reinterpret_cast<const char*>(src) + off, 16);
                }
            } else {
#pragma unroll
                for (int c = 0; c < CPT; ++c)
                    if (j0 + c < nx) cp_async_n(dst + c, src + c, (int)sizeof(T));
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int s = 0; s < PF - 1; ++s) issue(s, s);
    for (int i0 = 0; i0 < nt; i0 += PF) {
#pragma unroll
        for (int s = 0; s < PF; ++s) {
            const int i = i0 + s;
            if (i >= nt) break;
            issue(i + PF - 1, (s + PF - 1) % PF);
            cp_async_wait<PF - 1>();  // this thread's copy of row i has landed
            const T* rrow = ring + s * nx;
            T* cur = buf + (i & 1) * nx;
            const T* prv = buf + ((i & 1) ^ 1) * nx;
            if (active) {
                Chunk<T, CPT> rhs;
                if constexpr (VEC) {
                    rhs = *reinterpret_cast<const Chunk<T, CPT>*>(rrow + j0);
                } else {
#pragma unroll
                    for (int c = 0; c < CPT; ++c) rhs.v[c] = j0 + c < nx ? rrow[j0 + c] : T(0);
                }
                Chunk<T, CPT> out;
                if (i == 0) {
#pragma unroll
                    for (int c = 0; c < CPT; ++c) out.v[c] = rhs.v[c];
                } else {
                    const T left = prv[jl];
                    const T right = prv[jr];
#pragma unroll
                    for (int c = 0; c < CPT; ++c) {
                        const T xm = c == 0 ? left : d1[c - 1];
                        const T xp = c == CPT - 1 ? right : d1[c + 1];
                        const T tprev = (i == 1) ? d1[c] : T(2) * d1[c] - d2[c];
                        out.v[c] = g.dt2 * rhs.v[c] + tprev +
                                   g.lam2 * (kxm[c] * xm - ktm[c] * d1[c] + kxp[c] * xp);
                    }
                }
                if constexpr (VEC) {
                    *reinterpret_cast<Chunk<T, CPT>*>(x + (int64_t)i * nx + j0) = out;
                    *reinterpret_cast<Chunk<T, CPT>*>(cur + j0) = out;
                } else {
#pragma unroll
                    for (int c = 0; c < CPT; ++c) {
                        if (j0 + c < nx) {
                            x[(int64_t)i * nx + j0 + c] = out.v[c];
                            cur[j0 + c] = out.v[c];
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < CPT; ++c) {
                    d2[c] = d1[c];
                    d1[c] = out.v[c];
                }
            }
            __syncthreads();
        }
    }
    cp_async_wait<0>();
}

template <typename T, int CPT, int PF, bool VEC>
__global__ void __launch_bounds__(1024) wave_march_kernel(WaveDev<T> g, const T* __restrict__ b,
                                                          T* __restrict__ x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    march_instance<T, CPT, PF, VEC>(g, b, x, smem_raw);
}


}  // namespace wavedev
}  // namespace odil
