// L-BFGS in the compact representation (Byrd, Nocedal and Schnabel 1994;
// Nocedal & Wright eq. 7.24) with its small algebra on the device, so that
// an iteration whose first trial step satisfies the Wolfe conditions needs
// no host round trip but the one read of its status.  Replaces the host side
// of the reference's L-BFGS driver (optimizer.py:61-99: scipy's
// fmin_l_bfgs_b, m = 50, maxls = 50, pgtol = 1e-16, factr = 0, no bounds).
//
// Device state (caller-owned):
//   ring  int32[4]: [0] k pairs held, [1] head (slot of the oldest pair),
//         [2] m, [3] slot written by the last update (-1: none)
//   SY, YY  FP64[m][m] by slot: SY[a][b] = s_a . y_b, YY[a][b] = y_a . y_b
//   dg    FP64[2m]: dg[2 j] = s_j . g, dg[2 j + 1] = y_j . g at the iterate
//   sc    FP64[16]: [0] f, [1] gamma, [2] phi'(0) = g . d, [3] trial step,
//         [4] f at the trial, [5] phi'(step) = g_trial . d, [6] status
//         (0 accepted, 1 rejected: the host line search takes over,
//         2 d is not a descent direction), [7] c1, [8] c2, [9] eps (the
//         approximate-Wolfe tolerance of phi(0) relative), [10] first-step
//         flag (1: the trial is the steepest-descent step min(1, 1/|g|))
// Pairs: rows 2 j (s_j) and 2 j + 1 (y_j) of H [2m][n]; the pair of order
// c (0 = oldest) lives in slot (head + c) mod m.
#include "common.cuh"

namespace odil {
namespace {

constexpr int LT = 256;
constexpr int kMaxM = 128;

// coef[gidx + 1] of d = sum_{row < gidx} coef[row] H[row] + coef[gidx] g =
// -H_k g; gidx (even, 2 <= gidx <= 2m) covers every held slot.
//
// The k x k block R = S^T Y of the held pairs, in pair order, is staged in
// shared memory (row stride k | 1, odd, so the column reads of warp 0 spread
// over the banks) by the whole block, each thread issuing all of its loads
// before its stores.  The two triangular solves are right-looking on warp 0:
// lane l keeps the running right-hand sides of pairs l, l + 32, l + 64,
// l + 96 in registers; per pair the owner's value times the stored
// reciprocal of the diagonal is shuffled to every lane, which subtracts its
// multiple -- one shuffle and one multiply-add on the dependency chain per
// pair instead of a warp reduction.  The product with Y^T Y in between is
// spread over all warps.
constexpr int CT = 256;
constexpr int CQ = kMaxM / 32;

__host__ __device__ __forceinline__ int coef_ld(int k) { return k | 1; }

// x <- R^-1 x (kTrans = false, R upper) or R^-T x (kTrans = true) on one
// warp; x[q] holds the entry of pair 32 q + lane.
template <bool kTrans>
__device__ __forceinline__ void coef_trsv(const double* __restrict__ R, int ld,
                                          const double* __restrict__ rinv, int k, int lane,
                                          double (&x)[CQ]) {
    if (!kTrans) {
        // Backward: pair r from k-1 down; rows c < r lose R[c][r] x[r].
#pragma unroll
        for (int qb = CQ - 1; qb >= 0; --qb) {
            for (int rr = 31; rr >= 0; --rr) {
                const int r = 32 * qb + rr;
                if (r >= k) continue;
                const double xr = __shfl_sync(0xffffffffu, x[qb], rr) * rinv[r];
                if (lane == rr) x[qb] = xr;
#pragma unroll
                for (int q = 0; q <= qb; ++q) {
                    const int c = 32 * q + lane;
                    if (c < r) x[q] = fma(-R[c * ld + r], xr, x[q]);
                }
            }
        }
    } else {
        // Forward with R^T: pair r from 0 up; rows c > r lose R[r][c] x[r].
#pragma unroll
        for (int qb = 0; qb < CQ; ++qb) {
            for (int rr = 0; rr < 32; ++rr) {
                const int r = 32 * qb + rr;
                if (r >= k) break;
                const double xr = __shfl_sync(0xffffffffu, x[qb], rr) * rinv[r];
                if (lane == rr) x[qb] = xr;
#pragma unroll
                for (int q = qb; q < CQ; ++q) {
                    const int c = 32 * q + lane;
                    if (c > r && c < k) x[q] = fma(-R[r * ld + c], xr, x[q]);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(CT) lbfgs_coef_kernel(int mcap, int gidx,
                                                        const int* __restrict__ ring,
                                                        const double* __restrict__ SY,
                                                        const double* __restrict__ YY,
                                                        const double* __restrict__ dg,
                                                        const double* __restrict__ sc,
                                                        double* __restrict__ coef) {
    extern __shared__ double Rs[];  // [k][coef_ld(k)], R in pair order
    __shared__ double b[kMaxM], t[kMaxM], w[kMaxM], rinv[kMaxM];
    __shared__ int slot[kMaxM];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k = ring[0], head = ring[1], m = ring[2];
    for (int r = tid; r <= gidx; r += CT) coef[r] = 0.0;
    __syncthreads();
    // No pair held: steepest descent.  The shared block is sized for mcap
    // pairs; a ring that does not match (not reachable through the
    // optimizer) takes the same fallback.
    if (k <= 0 || m != mcap || k > m || head < 0 || head >= m) {
        if (tid == 0) coef[gidx] = -1.0;
        return;
    }
    const double gamma = sc[1];
    const int ld = coef_ld(k);
    for (int c = tid; c < k; c += CT) slot[c] = (head + c) % m;
    __syncthreads();
    for (int e0 = tid; e0 < k * k; e0 += 8 * CT) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = e0 + u * CT;
            const int r = e / k, c = e - r * k;
            v[u] = e < k * k ? SY[slot[r] * m + slot[c]] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = e0 + u * CT;
            const int r = e / k, c = e - r * k;
            if (e < k * k) Rs[r * ld + c] = v[u];
        }
    }
    for (int c = tid; c < k; c += CT) b[c] = dg[2 * slot[c] + 1];
    __syncthreads();
    for (int c = tid; c < k; c += CT) rinv[c] = 1.0 / Rs[c * ld + c];
    __syncthreads();
    // t = R^-1 a, a = S^T g in pair order.
    if (warp == 0) {
        double x[CQ];
#pragma unroll
        for (int q = 0; q < CQ; ++q) {
            const int c = 32 * q + lane;
            x[q] = c < k ? dg[2 * slot[c]] : 0.0;
        }
        coef_trsv<false>(Rs, ld, rinv, k, lane, x);
#pragma unroll
        for (int q = 0; q < CQ; ++q) {
            const int c = 32 * q + lane;
            if (c < k) t[c] = x[q];
        }
    }
    __syncthreads();
    // w = (D + gamma Y^T Y) t - gamma b: one warp per pair c, lanes over e,
    // four pairs per warp with all their loads in flight together.
    constexpr int CW = CT / 32;
    for (int cq = warp; cq < k; cq += 4 * CW) {
        double v[4][CQ];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int c = cq + i * CW;
#pragma unroll
            for (int q = 0; q < CQ; ++q) {
                const int e = 32 * q + lane;
                v[i][q] = (c < k && e < k) ? YY[(int64_t)slot[c] * m + slot[e]] : 0.0;
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int c = cq + i * CW;
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < CQ; ++q) {
                const int e = 32 * q + lane;
                if (e < k) s = fma(v[i][q], t[e], s);
            }
            s = warp_sum(s);
            if (lane == 0 && c < k) w[c] = Rs[c * ld + c] * t[c] + gamma * s - gamma * b[c];
        }
    }
    __syncthreads();
    // p = R^-T w; coef of s_c is -p_c, of y_c gamma t_c.
    if (warp == 0) {
        double x[CQ];
#pragma unroll
        for (int q = 0; q < CQ; ++q) {
            const int c = 32 * q + lane;
            x[q] = c < k ? w[c] : 0.0;
        }
        coef_trsv<true>(Rs, ld, rinv, k, lane, x);
#pragma unroll
        for (int q = 0; q < CQ; ++q) {
            const int c = 32 * q + lane;
            if (c < k && 2 * slot[c] + 1 < gidx) {
                coef[2 * slot[c]] = -x[q];
                coef[2 * slot[c] + 1] = gamma * t[c];
            }
        }
        if (lane == 0) coef[gidx] = -gamma;
    }
}

// Dynamic shared memory of lbfgs_coef_kernel for up to m held pairs.
inline size_t coef_smem(int m) { return (size_t)m * coef_ld(m) * sizeof(double); }

// xt = x + a d with the trial step a chosen on the device from phi'(0) =
// dots[0]: the steepest-descent step min(1, 1/|g|) while no pair is held,
// else 1.  Block 0 records phi'(0) and a.
template <typename T>
__global__ void __launch_bounds__(LT) lbfgs_trial_kernel(int64_t n, T* __restrict__ xt,
                                                         const T* __restrict__ x,
                                                         const T* __restrict__ d,
                                                         const double* __restrict__ dots,
                                                         const int* __restrict__ ring,
                                                         double* __restrict__ sc) {
    const double dphi0 = dots[0];
    double a = 1.0;
    if (ring[0] == 0) {
        const double gn = sqrt(fmax(-dphi0, 0.0));
        a = fmin(1.0, 1.0 / fmax(gn, 1e-300));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc[2] = dphi0;
        sc[3] = a;
        sc[10] = ring[0] == 0 ? 1.0 : 0.0;
    }
    const T at = (T)a;
    const int64_t stride = (int64_t)gridDim.x * LT;
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < n; i += stride)
        xt[i] = x[i] + at * d[i];
}

// Status of a trial: 0 accepted, 1 rejected, 2 d is not a descent direction.
__device__ __forceinline__ double wolfe_status(const double* sc, double fa, double dpa) {
    const double f0 = sc[0], dphi0 = sc[2], a = sc[3], c1 = sc[7], c2 = sc[8];
    const double eps = sc[9] * fabs(f0);
    if (!(dphi0 < 0.0)) return 2.0;
    if (!isfinite(fa) || !isfinite(dpa) || dpa < c2 * dphi0) return 1.0;
    if (fa <= f0 + c1 * a * dphi0) return 0.0;
    if (fa <= f0 + eps && dpa <= (2.0 * c1 - 1.0) * dphi0) return 0.0;
    return 1.0;
}

// The Wolfe test of the trial (phi(a) <= phi(0) + c1 a phi'(0) and phi'(a) >=
// c2 phi'(0)), or the approximate Wolfe conditions of Hager and Zhang
// (phi(a) <= phi(0) + eps |phi(0)|, c2 phi'(0) <= phi'(a) <= (2 c1 - 1)
// phi'(0)), as the host line search accepts a step.
__global__ void lbfgs_accept_kernel(const double* __restrict__ ft,
                                    const double* __restrict__ dpa_dots,
                                    double* __restrict__ sc) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double fa = ft[0], dpa = dpa_dots[0];
    sc[4] = fa;
    sc[5] = dpa;
    sc[6] = wolfe_status(sc, fa, dpa);
}

// The new pair s = a d, y = g_trial - g into rows 0 and 1 of sy (accepted
// trials only).
template <typename T>
__global__ void __launch_bounds__(LT) lbfgs_pair_kernel(int64_t n, T* __restrict__ sy,
                                                        const T* __restrict__ d,
                                                        const T* __restrict__ gt,
                                                        const T* __restrict__ g,
                                                        const double* __restrict__ sc) {
    if (sc[6] != 0.0) return;
    const T a = (T)sc[3];
    const int64_t stride = (int64_t)gridDim.x * LT;
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < n; i += stride) {
        sy[i] = a * d[i];
        sy[n + i] = gt[i] - g[i];
    }
}

// The pair, its dots and the Wolfe test in one pass over d, g_trial and g:
// s = a d and y = g_trial - g into sy (scratch: written whatever the test
// decides), and the five dots g_trial.d, s.y, s.g_trial, y.y, y.g_trial
// (per-thread sums in the working precision, FP64 partials per block, stored
// dot-major).  The last block adds each dot's partials in index order, then
// mode 0: the test of lbfgs_accept_kernel on f(trial) = ft[0] and
// phi'(a) = g_trial.d; mode 1: the host line search chose the step (sc[3],
// sc[4], sc[6] = 0 set by the host), nothing is tested.  Q = [[s.y, s.gt],
// [y.y, y.gt]] for the update.  Replaces the g_trial.d multi-dot, the accept
// and pair kernels and the 2 x 2 multi-dot of the unfused iteration.
constexpr int PD = 5;


template <typename T>
__global__ void __launch_bounds__(LT) lbfgs_pair_dots_kernel(
    int64_t n, T* __restrict__ sy, const T* __restrict__ d, const T* __restrict__ gt,
    const T* __restrict__ g, const double* __restrict__ ft, int mode, double* __restrict__ sc,
    double* __restrict__ Q, ReduceWs ws) {
    const T a = (T)sc[3];
    T acc[PD];
#pragma unroll
    for (int j = 0; j < PD; ++j) acc[j] = T(0);
    const int64_t stride = (int64_t)gridDim.x * LT;
    auto step = [&](T dv, T gtv, T gv, int64_t i) {
        const T sv = a * dv, yv = gtv - gv;
        sy[i] = sv;
        sy[n + i] = yv;
        acc[0] += gtv * dv;
        acc[1] += sv * yv;
        acc[2] += sv * gtv;
        acc[3] += yv * yv;
        acc[4] += yv * gtv;
    };
    // PU elements per thread per pass, all their loads issued first.
    constexpr int PU = 4;
    int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x;
    for (; i + (PU - 1) * stride < n; i += PU * stride) {
        T dv[PU], gtv[PU], gv[PU];
#pragma unroll
        for (int u = 0; u < PU; ++u) {
            dv[u] = d[i + u * stride];
            gtv[u] = gt[i + u * stride];
            gv[u] = g[i + u * stride];
        }
#pragma unroll
        for (int u = 0; u < PU; ++u) step(dv[u], gtv[u], gv[u], i + u * stride);
    }
    for (; i < n; i += stride) step(d[i], gt[i], g[i], i);
    __shared__ double red[LT / 32][PD];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < PD; ++j) {
        const double v = warp_sum((double)acc[j]);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    const int64_t nb = gridDim.x;
    if (threadIdx.x < PD) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < LT / 32; ++w) v += red[w][threadIdx.x];
        ws.partials[threadIdx.x * nb + blockIdx.x] = v;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(ws.counter, 1u);
        is_last = prev == (unsigned)(nb - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // All five sums in one pass over the block partials (fixed order).
    double accp[PD];
#pragma unroll
    for (int j = 0; j < PD; ++j) accp[j] = 0.0;
    for (int64_t q = threadIdx.x; q < nb; q += LT) {
#pragma unroll
        for (int j = 0; j < PD; ++j) accp[j] += __ldcg(ws.partials + j * nb + q);
    }
#pragma unroll
    for (int j = 0; j < PD; ++j) {
        const double v = warp_sum(accp[j]);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    __shared__ double tot[PD];
    if (threadIdx.x < PD) {
        double v = 0.0;
#pragma unroll
        for (int w = 0; w < LT / 32; ++w) v += red[w][threadIdx.x];
        tot[threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (mode == 0) {
            const double fa = ft[0], dpa = tot[0];
            sc[4] = fa;
            sc[5] = dpa;
            sc[6] = wolfe_status(sc, fa, dpa);
        } else {
            sc[5] = tot[0];
        }
        Q[0] = tot[1];
        Q[1] = tot[2];
        Q[2] = tot[3];
        Q[3] = tot[4];
        *ws.counter = 0u;
    }
}

// Ring and matrix update after an accepted step.  P: [rows][3] dots of the
// stored rows with (g_trial, s, y); Q: [2][2] = [[s.y, s.g_trial],
// [y.y, y.g_trial]].  The pair is kept when s.y > 1e-12 y.y (the curvature
// condition, as the host version); the dots with g_trial become dg.
__global__ void __launch_bounds__(32) lbfgs_update_kernel(int* __restrict__ ring,
                                                          double* __restrict__ SY,
                                                          double* __restrict__ YY,
                                                          double* __restrict__ dg,
                                                          double* __restrict__ sc,
                                                          const double* __restrict__ P, int rows,
                                                          const double* __restrict__ Q) {
    __shared__ int s_slot;
    const int lane = threadIdx.x;
    if (sc[6] != 0.0) return;
    const int k = ring[0], head = ring[1], m = ring[2];
    const double sy = Q[0], sgt = Q[1], yy = Q[2], ygt = Q[3];
    // dots of the held pairs with the new gradient
    for (int r = lane; r < 2 * m; r += 32) dg[r] = r < rows ? P[r * 3] : 0.0;
    __syncwarp();
    if (lane == 0) {
        s_slot = -1;
        if (isfinite(sy) && isfinite(yy) && sy > 1e-12 * yy) {
            int slot;
            if (k < m) {
                slot = (head + k) % m;
                ring[0] = k + 1;
            } else {
                slot = head;
                ring[1] = (head + 1) % m;
            }
            s_slot = slot;
            sc[1] = sy / yy;
        }
        ring[3] = s_slot;
        sc[0] = sc[4];
    }
    __syncwarp();
    const int slot = s_slot;
    if (slot < 0) return;
    const int k2 = ring[0], head2 = ring[1];
    for (int c = lane; c < k2; c += 32) {
        const int j = (head2 + c) % m;
        if (j == slot) continue;
        SY[slot * m + j] = P[(2 * j + 1) * 3 + 1];  // s_new . y_j
        SY[j * m + slot] = P[(2 * j) * 3 + 2];      // s_j . y_new
        const double v = P[(2 * j + 1) * 3 + 2];    // y_j . y_new
        YY[slot * m + j] = v;
        YY[j * m + slot] = v;
    }
    if (lane == 0) {
        SY[slot * m + slot] = sy;
        YY[slot * m + slot] = yy;
        dg[2 * slot] = sgt;
        dg[2 * slot + 1] = ygt;
    }
}

// Accepted step only: H rows of the slot written by the last update <-
// (s, y) (when the pair was kept), and g <- g_trial (when g is given).
template <typename T>
__global__ void __launch_bounds__(LT) lbfgs_commit_kernel(int64_t n, T* __restrict__ H, int64_t ld,
                                                          const T* __restrict__ sy,
                                                          T* __restrict__ g,
                                                          const T* __restrict__ gt,
                                                          const int* __restrict__ ring,
                                                          const double* __restrict__ sc) {
    if (sc[6] != 0.0) return;
    const int slot = ring[3];
    T* hs = slot >= 0 ? H + (int64_t)(2 * slot) * ld : nullptr;
    const int64_t stride = (int64_t)gridDim.x * LT;
    for (int64_t i = (int64_t)blockIdx.x * LT + threadIdx.x; i < n; i += stride) {
        if (hs) {
            hs[i] = sy[i];
            hs[ld + i] = sy[n + i];
        }
        if (g) g[i] = gt[i];
    }
}

inline unsigned lgrid(int64_t n) {
    int64_t b = (n + LT - 1) / LT;
    const int64_t cap = 152 * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <typename T>
int trial_impl(int64_t n, T* xt, const T* x, const T* d, const double* dots, const int* ring,
               double* sc, void* stream) {
    if (n < 1) return ODIL_ERR_SHAPE;
    if (!xt || !x || !d || !dots || !ring || !sc) return ODIL_ERR_ARG;
    lbfgs_trial_kernel<T><<<lgrid(n), LT, 0, as_stream(stream)>>>(n, xt, x, d, dots, ring, sc);
    return launch_status();
}

template <typename T>
int pair_impl(int64_t n, T* sy, const T* d, const T* gt, const T* g, const double* sc,
              void* stream) {
    if (n < 1) return ODIL_ERR_SHAPE;
    if (!sy || !d || !gt || !g || !sc) return ODIL_ERR_ARG;
    lbfgs_pair_kernel<T><<<lgrid(n), LT, 0, as_stream(stream)>>>(n, sy, d, gt, g, sc);
    return launch_status();
}

// Blocks of the pair-and-dots pass: at most 2 per SM, so the FP64 warp
// reductions of the five dots (GB300's FP64 pipe is narrow) are paid by few
// blocks, each streaming a long stretch.
inline unsigned pd_grid(int64_t n) {
    int64_t b = (n + LT - 1) / LT;
    const int64_t cap = 152 * 2;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <typename T>
int pair_dots_impl(int64_t n, T* sy, const T* d, const T* gt, const T* g, const double* ft,
                   int mode, double* sc, double* Q, void* ws, int64_t ws_bytes, void* stream) {
    if (n < 1) return ODIL_ERR_SHAPE;
    if (mode != 0 && mode != 1) return ODIL_ERR_ARG;
    if (!sy || !d || !gt || !g || !sc || !Q || (mode == 0 && !ft)) return ODIL_ERR_ARG;
    const unsigned blocks = pd_grid(n);
    if (!ws || ws_bytes < kReduceHeader + (int64_t)PD * blocks * (int64_t)sizeof(double))
        return ODIL_ERR_WORKSPACE;
    lbfgs_pair_dots_kernel<T><<<blocks, LT, 0, as_stream(stream)>>>(n, sy, d, gt, g, ft, mode, sc,
                                                                   Q, reduce_ws(ws));
    return launch_status();
}

template <typename T>
int commit_impl(int64_t n, T* H, int64_t ld, const T* sy, T* g, const T* gt, const int* ring,
                const double* sc, void* stream) {
    if (n < 1 || ld < n) return ODIL_ERR_SHAPE;
    if (!H || !sy || !ring || !sc || (g && !gt)) return ODIL_ERR_ARG;
    lbfgs_commit_kernel<T><<<lgrid(n), LT, 0, as_stream(stream)>>>(n, H, ld, sy, g, gt, ring, sc);
    return launch_status();
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_lbfgs_coef(int32_t m, int32_t gidx, const int* ring, const double* SY,
                             const double* YY, const double* dg, const double* sc, double* coef,
                             void* stream) {
    if (m < 1 || m > kMaxM || gidx < 2 || gidx > 2 * m || gidx % 2) return ODIL_ERR_SHAPE;
    if (!ring || !SY || !YY || !dg || !sc || !coef) return ODIL_ERR_ARG;
    const size_t smem = coef_smem(m);
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(
            lbfgs_coef_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return ODIL_ERR_LAUNCH;
    }
    lbfgs_coef_kernel<<<1, CT, smem, as_stream(stream)>>>(m, gidx, ring, SY, YY, dg, sc, coef);
    return launch_status();
}

ODIL_API int odil_lbfgs_trial_f32(int64_t n, float* xt, const float* x, const float* d,
                                  const double* dots, const int* ring, double* sc, void* stream) {
    return trial_impl<float>(n, xt, x, d, dots, ring, sc, stream);
}
ODIL_API int odil_lbfgs_trial_f64(int64_t n, double* xt, const double* x, const double* d,
                                  const double* dots, const int* ring, double* sc, void* stream) {
    return trial_impl<double>(n, xt, x, d, dots, ring, sc, stream);
}

ODIL_API int odil_lbfgs_accept(const double* ft, const double* dpa, double* sc, void* stream) {
    if (!ft || !dpa || !sc) return ODIL_ERR_ARG;
    lbfgs_accept_kernel<<<1, 32, 0, as_stream(stream)>>>(ft, dpa, sc);
    return launch_status();
}

ODIL_API int odil_lbfgs_pair_f32(int64_t n, float* sy, const float* d, const float* gt,
                                 const float* g, const double* sc, void* stream) {
    return pair_impl<float>(n, sy, d, gt, g, sc, stream);
}
ODIL_API int odil_lbfgs_pair_f64(int64_t n, double* sy, const double* d, const double* gt,
                                 const double* g, const double* sc, void* stream) {
    return pair_impl<double>(n, sy, d, gt, g, sc, stream);
}

ODIL_API int64_t odil_lbfgs_pair_dots_workspace_bytes(int64_t n) {
    if (n < 1) return 0;
    return kReduceHeader + (int64_t)PD * pd_grid(n) * (int64_t)sizeof(double);
}
ODIL_API int odil_lbfgs_pair_dots_f32(int64_t n, float* sy, const float* d, const float* gt,
                                      const float* g, const double* ft, int32_t mode, double* sc,
                                      double* Q, void* workspace, int64_t workspace_bytes,
                                      void* stream) {
    return pair_dots_impl<float>(n, sy, d, gt, g, ft, mode, sc, Q, workspace, workspace_bytes,
                                 stream);
}
ODIL_API int odil_lbfgs_pair_dots_f64(int64_t n, double* sy, const double* d, const double* gt,
                                      const double* g, const double* ft, int32_t mode,
                                      double* sc, double* Q, void* workspace,
                                      int64_t workspace_bytes, void* stream) {
    return pair_dots_impl<double>(n, sy, d, gt, g, ft, mode, sc, Q, workspace, workspace_bytes,
                                  stream);
}

ODIL_API int odil_lbfgs_update(int* ring, double* SY, double* YY, double* dg, double* sc,
                               const double* P, int32_t rows, const double* Q, void* stream) {
    if (rows < 0) return ODIL_ERR_SHAPE;
    if (!ring || !SY || !YY || !dg || !sc || !Q || (rows > 0 && !P)) return ODIL_ERR_ARG;
    lbfgs_update_kernel<<<1, 32, 0, as_stream(stream)>>>(ring, SY, YY, dg, sc, P, rows, Q);
    return launch_status();
}

ODIL_API int odil_lbfgs_commit_f32(int64_t n, float* H, int64_t ld, const float* sy, float* g,
                                   const float* gt, const int* ring, const double* sc,
                                   void* stream) {
    return commit_impl<float>(n, H, ld, sy, g, gt, ring, sc, stream);
}
ODIL_API int odil_lbfgs_commit_f64(int64_t n, double* H, int64_t ld, const double* sy, double* g,
                                   const double* gt, const int* ring, const double* sc,
                                   void* stream) {
    return commit_impl<double>(n, H, ld, sy, g, gt, ring, sc, stream);
}
