// Geometric multigrid for the normal equations of the lid-driven cavity
// (Newton / Gauss-Newton steps of ns_steady.py solved as util.py:509-604
// solves them: J^T J d = -J^T f with V-cycles on J^T J), cell-centred:
//
//   * fine level: J^T J applied matrix-free from the Jacobian's coefficient
//     fields (the [neq][15][n][n] output of odil_ns_jacobian_*; 5-point
//     stencils per (equation, field)): w = J x, then y = J^T w;
//   * J^T J as explicit 25-point stencils per (field, field) block, the
//     input of the Galerkin product (only the 13 points with |dx|+|dy| <= 2
//     are nonzero on the fine level);
//   * coarse levels: Galerkin R A P with bilinear cell-centred prolongation P
//     (weights 3/4, 1/4 per axis; at a wall the outer weight goes to the
//     wall cell) and R = P^T / 4; the coarse stencils stay 25-point;
//   * smoothing: damped block Jacobi on the 3 x 3 per-cell blocks;
//   * coarsest level: dense FP64 inverse (Gauss-Jordan in one block).
//
// Layouts: a vector is [3][n][n] (u, v, p), cell (i, j) at i * n + j with i
// along x; a 25-point operator is [9][25][n][n], block (f, g) = 3 f + g,
// point d = (dx + 2) * 5 + (dy + 2), (A x)_f[c] = sum_g sum_d A[fg][d][c]
// x_g[c + d], points outside the grid skipped; Dinv is [9][n][n].
#include "common.cuh"

namespace odil {
namespace {

constexpr int MT = 256;
// The Jacobian's shift index s (stencil_var order of ns_steady.py:154-163):
// (0, 0), (-1, 0), (1, 0), (0, -1), (0, 1).  Constant after unrolling.
__host__ __device__ __forceinline__ constexpr int shx(int s) { return s == 1 ? -1 : (s == 2 ? 1 : 0); }
__host__ __device__ __forceinline__ constexpr int shy(int s) { return s == 3 ? -1 : (s == 4 ? 1 : 0); }

inline unsigned nblocks(int64_t n) {
    int64_t b = (n + MT - 1) / MT;
    return (unsigned)(b < 1 ? 1 : b);
}

// w_e = sum_f sum_s C[e][5 f + s][c] x_f[c + s]   (J x, one thread per cell)
template <typename T>
__global__ void __launch_bounds__(MT) jx_kernel(int n, int neq, const T* __restrict__ C,
                                                const T* __restrict__ x, T* __restrict__ w) {
    const int64_t N = (int64_t)n * n;
    const int64_t c = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (c >= N) return;
    const int i = (int)(c / n), j = (int)(c % n);
    T xs[3][5];
#pragma unroll
    for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            const int ii = i + shx(s), jj = j + shy(s);
            xs[f][s] = (ii >= 0 && ii < n && jj >= 0 && jj < n)
                           ? __ldg(x + f * N + (int64_t)ii * n + jj)
                           : T(0);
        }
    for (int e = 0; e < neq; ++e) {
        const T* Ce = C + (int64_t)e * 15 * N + c;
        T acc = T(0);
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int s = 0; s < 5; ++s) acc += __ldg(Ce + (5 * f + s) * N) * xs[f][s];
        w[(int64_t)e * N + c] = acc;
    }
}

// y_f[c] = sum_e sum_s C[e][5 f + s][c - s] w_e[c - s]   (J^T w), then
// mode 0: out = y; 1: out = b - y; 2: out = x + omega Dinv (b - y).
template <typename T>
__global__ void __launch_bounds__(MT) jtw_kernel(int n, int neq, const T* __restrict__ C,
                                                 const T* __restrict__ w, const T* __restrict__ b,
                                                 const T* __restrict__ x,
                                                 const T* __restrict__ Dinv, T* __restrict__ out,
                                                 T omega, int mode) {
    const int64_t N = (int64_t)n * n;
    const int64_t c = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (c >= N) return;
    const int i = (int)(c / n), j = (int)(c % n);
    T y[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        const int ii = i - shx(s), jj = j - shy(s);
        if (ii < 0 || ii >= n || jj < 0 || jj >= n) continue;
        const int64_t r = (int64_t)ii * n + jj;
        for (int e = 0; e < neq; ++e) {
            const T we = __ldg(w + (int64_t)e * N + r);
            const T* Ce = C + (int64_t)e * 15 * N + r;
#pragma unroll
            for (int f = 0; f < 3; ++f) y[f] += __ldg(Ce + (5 * f + s) * N) * we;
        }
    }
    if (mode == 0) {
#pragma unroll
        for (int f = 0; f < 3; ++f) out[f * N + c] = y[f];
        return;
    }
    T r[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) r[f] = __ldg(b + f * N + c) - y[f];
    if (mode == 1) {
#pragma unroll
        for (int f = 0; f < 3; ++f) out[f * N + c] = r[f];
        return;
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        T d = T(0);
#pragma unroll
        for (int g = 0; g < 3; ++g) d += __ldg(Dinv + (3 * f + g) * N + c) * r[g];
        out[f * N + c] = __ldg(x + f * N + c) + omega * d;
    }
}

// Explicit J^T J as 25-point stencils: A[fg][d][c] = sum_e sum_{s1, s2:
// s2 - s1 = d} C[e][5 f + s1][c - s1] C[e][5 g + s2][c - s1].  One thread
// per (cell, block).
__global__ void __launch_bounds__(MT) fine_ata_kernel(int n, int neq, const float* __restrict__ C,
                                                      float* __restrict__ A) {
    const int64_t N = (int64_t)n * n;
    const int64_t t = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (t >= 9 * N) return;
    const int fg = (int)(t / N);
    const int64_t c = t % N;
    const int f = fg / 3, g = fg % 3;
    const int i = (int)(c / n), j = (int)(c % n);
    float acc[25];
#pragma unroll
    for (int d = 0; d < 25; ++d) acc[d] = 0.f;
#pragma unroll
    for (int s1 = 0; s1 < 5; ++s1) {
        const int ri = i - shx(s1), rj = j - shy(s1);
        if (ri < 0 || ri >= n || rj < 0 || rj >= n) continue;
        const int64_t r = (int64_t)ri * n + rj;
        for (int e = 0; e < neq; ++e) {
            const float* Ce = C + (int64_t)e * 15 * N + r;
            const float a = __ldg(Ce + (5 * f + s1) * N);
            if (a == 0.f) continue;
#pragma unroll
            for (int s2 = 0; s2 < 5; ++s2) {
                const int ti = ri + shx(s2), tj = rj + shy(s2);
                if (ti < 0 || ti >= n || tj < 0 || tj >= n) continue;
                const int d = (shx(s2) - shx(s1) + 2) * 5 + (shy(s2) - shy(s1) + 2);
                acc[d] += a * __ldg(Ce + (5 * g + s2) * N);
            }
        }
    }
    float* Ab = A + (int64_t)fg * 25 * N + c;
#pragma unroll
    for (int d = 0; d < 25; ++d) Ab[d * N] = acc[d];
}

// Inverse of the 3 x 3 diagonal block of every cell (the centre point of the
// nine blocks), in FP64; a singular block gives the inverse of its diagonal
// (zero where the diagonal is zero).
__global__ void __launch_bounds__(MT) dinv_kernel(int n, const float* __restrict__ A,
                                                  float* __restrict__ Dinv) {
    const int64_t N = (int64_t)n * n;
    const int64_t c = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (c >= N) return;
    double m[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m[k] = (double)__ldg(A + ((int64_t)k * 25 + 12) * N + c);
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c01 = m[5] * m[6] - m[3] * m[8];
    const double c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    const double scale = fabs(m[0]) + fabs(m[4]) + fabs(m[8]);
    double inv[9];
    if (fabs(det) > 1e-12 * scale * scale * scale && isfinite(det)) {
        const double id = 1.0 / det;
        inv[0] = c00 * id;
        inv[1] = (m[2] * m[7] - m[1] * m[8]) * id;
        inv[2] = (m[1] * m[5] - m[2] * m[4]) * id;
        inv[3] = c01 * id;
        inv[4] = (m[0] * m[8] - m[2] * m[6]) * id;
        inv[5] = (m[2] * m[3] - m[0] * m[5]) * id;
        inv[6] = c02 * id;
        inv[7] = (m[1] * m[6] - m[0] * m[7]) * id;
        inv[8] = (m[0] * m[4] - m[1] * m[3]) * id;
    } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) inv[k] = 0.0;
        inv[0] = m[0] != 0.0 ? 1.0 / m[0] : 0.0;
        inv[4] = m[4] != 0.0 ? 1.0 / m[4] : 0.0;
        inv[8] = m[8] != 0.0 ? 1.0 / m[8] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) Dinv[(int64_t)k * N + c] = (float)inv[k];
}

// Weight of coarse cell C in row i of the 1D cell-centred prolongation on a
// fine axis of 2 nc cells: primary parent i / 2 (3/4), secondary parent
// i / 2 -+ 1 (1/4) toward the fine cell's side; at a wall the missing
// secondary's weight goes to the primary (1).
__device__ __forceinline__ float pw(int i, int C, int nc) {
    const int c0 = i >> 1;
    const int c1 = (i & 1) ? c0 + 1 : c0 - 1;
    const bool has1 = c1 >= 0 && c1 < nc;
    if (C == c0) return has1 ? 0.75f : 1.0f;
    if (has1 && C == c1) return 0.25f;
    return 0.f;
}

// Galerkin product A_c = R A P, R = P^T / 4, 25-point in and out.  One
// thread per (coarse cell, block): 16 fine children x 25 points x 4 coarse
// targets, all unrolled, so the target of every product is a constant
// (the parents of fine cell 2 C + k are C + floor(k / 2) and its neighbour
// toward the odd side); walls only change weights (pw is 0 for a missing
// parent).
__global__ void __launch_bounds__(MT) galerkin_kernel(int n, const float* __restrict__ A,
                                                      float* __restrict__ Ac) {
    const int nc = n / 2;
    const int64_t N = (int64_t)n * n, Nc = (int64_t)nc * nc;
    const int64_t t = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (t >= 9 * Nc) return;
    const int fg = (int)(t / Nc);
    const int64_t cc = t % Nc;
    const int CI = (int)(cc / nc), CJ = (int)(cc % nc);
    float acc[25];
#pragma unroll
    for (int d = 0; d < 25; ++d) acc[d] = 0.f;
    const float* Ab = A + (int64_t)fg * 25 * N;
#pragma unroll
    for (int a = -1; a <= 2; ++a) {
        const int i = 2 * CI + a;
        const float ri = (i >= 0 && i < n) ? pw(i, CI, nc) : 0.f;
#pragma unroll
        for (int b = -1; b <= 2; ++b) {
            const int j = 2 * CJ + b;
            const float rj = (j >= 0 && j < n) ? pw(j, CJ, nc) : 0.f;
            const float rw = 0.25f * ri * rj;
            if (rw == 0.f) continue;
            const int64_t fi = (int64_t)i * n + j;
#pragma unroll
            for (int d = 0; d < 25; ++d) {
                const int dx = d / 5 - 2, dy = d % 5 - 2;
                const int ti = i + dx, tj = j + dy;
                if (ti < 0 || ti >= n || tj < 0 || tj >= n) continue;
                const float rv = rw * __ldg(Ab + (int64_t)d * N + fi);
                const int ki = a + dx, kj = b + dy;          // in [-3, 4]
                const int i0 = ki >> 1, i1 = (ki & 1) ? i0 + 1 : i0 - 1;
                const int j0 = kj >> 1, j1 = (kj & 1) ? j0 + 1 : j0 - 1;
                const float wi0 = pw(ti, CI + i0, nc), wi1 = pw(ti, CI + i1, nc);
                const float wj0 = pw(tj, CJ + j0, nc), wj1 = pw(tj, CJ + j1, nc);
                acc[(i0 + 2) * 5 + (j0 + 2)] += rv * wi0 * wj0;
                acc[(i0 + 2) * 5 + (j1 + 2)] += rv * wi0 * wj1;
                acc[(i1 + 2) * 5 + (j0 + 2)] += rv * wi1 * wj0;
                acc[(i1 + 2) * 5 + (j1 + 2)] += rv * wi1 * wj1;
            }
        }
    }
    float* Acb = Ac + (int64_t)fg * 25 * Nc + cc;
#pragma unroll
    for (int d = 0; d < 25; ++d) Acb[d * Nc] = acc[d];
}

// 25-point operator on a level: r_f = b_f - sum_g sum_d A[fg][d][c] x_g[c+d];
// mode 0: out = A x (b unused); 1: out = r; 2: out = x + omega Dinv r.
__global__ void __launch_bounds__(MT) smooth_kernel(int n, const float* __restrict__ A,
                                                    const float* __restrict__ Dinv,
                                                    const float* __restrict__ x,
                                                    const float* __restrict__ b,
                                                    float* __restrict__ out, float omega,
                                                    int mode) {
    const int64_t N = (int64_t)n * n;
    const int64_t c = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (c >= N) return;
    const int i = (int)(c / n), j = (int)(c % n);
    float y[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 25; ++d) {
        const int ti = i + d / 5 - 2, tj = j + d % 5 - 2;
        if (ti < 0 || ti >= n || tj < 0 || tj >= n) continue;
        const int64_t tc = (int64_t)ti * n + tj;
        const float x0 = __ldg(x + tc), x1 = __ldg(x + N + tc), x2 = __ldg(x + 2 * N + tc);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float* Af = A + ((int64_t)(3 * f) * 25 + d) * N + c;
            y[f] += __ldg(Af) * x0 + __ldg(Af + 25 * N) * x1 + __ldg(Af + 50 * N) * x2;
        }
    }
    if (mode == 0) {
#pragma unroll
        for (int f = 0; f < 3; ++f) out[f * N + c] = y[f];
        return;
    }
    float r[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) r[f] = __ldg(b + f * N + c) - y[f];
    if (mode == 1) {
#pragma unroll
        for (int f = 0; f < 3; ++f) out[f * N + c] = r[f];
        return;
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        float d = 0.f;
#pragma unroll
        for (int g = 0; g < 3; ++g) d += __ldg(Dinv + (3 * f + g) * N + c) * r[g];
        out[f * N + c] = __ldg(x + f * N + c) + omega * d;
    }
}

// out = omega Dinv b  (the first Jacobi sweep from x = 0)
__global__ void __launch_bounds__(MT) jacobi0_kernel(int64_t N, const float* __restrict__ Dinv,
                                                     const float* __restrict__ b,
                                                     float* __restrict__ out, float omega) {
    const int64_t c = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (c >= N) return;
    const float b0 = __ldg(b + c), b1 = __ldg(b + N + c), b2 = __ldg(b + 2 * N + c);
#pragma unroll
    for (int f = 0; f < 3; ++f)
        out[f * N + c] = omega * (__ldg(Dinv + (3 * f) * N + c) * b0 +
                                  __ldg(Dinv + (3 * f + 1) * N + c) * b1 +
                                  __ldg(Dinv + (3 * f + 2) * N + c) * b2);
}

// rc_f[C] = sum_i R(C, i) r_f[i], R = P^T / 4 (one thread per coarse cell)
__global__ void __launch_bounds__(MT) restrict_kernel(int n, const float* __restrict__ r,
                                                      float* __restrict__ rc) {
    const int nc = n / 2;
    const int64_t N = (int64_t)n * n, Nc = (int64_t)nc * nc;
    const int64_t cc = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (cc >= Nc) return;
    const int CI = (int)(cc / nc), CJ = (int)(cc % nc);
    float acc[3] = {0.f, 0.f, 0.f};
    for (int a = -1; a <= 2; ++a) {
        const int i = 2 * CI + a;
        if (i < 0 || i >= n) continue;
        const float wi = pw(i, CI, nc);
        if (wi == 0.f) continue;
        for (int b = -1; b <= 2; ++b) {
            const int j = 2 * CJ + b;
            if (j < 0 || j >= n) continue;
            const float w = 0.25f * wi * pw(j, CJ, nc);
            if (w == 0.f) continue;
            const int64_t fi = (int64_t)i * n + j;
#pragma unroll
            for (int f = 0; f < 3; ++f) acc[f] += w * __ldg(r + f * N + fi);
        }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) rc[f * Nc + cc] = acc[f];
}

// x_f[i] += sum_C P(i, C) e_f[C]  (one thread per fine cell)
__global__ void __launch_bounds__(MT) prolong_add_kernel(int n, const float* __restrict__ e,
                                                         float* __restrict__ x) {
    const int nc = n / 2;
    const int64_t N = (int64_t)n * n, Nc = (int64_t)nc * nc;
    const int64_t c = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (c >= N) return;
    const int i = (int)(c / n), j = (int)(c % n);
    const int pi0 = i >> 1, pi1 = (i & 1) ? pi0 + 1 : pi0 - 1;
    const int pj0 = j >> 1, pj1 = (j & 1) ? pj0 + 1 : pj0 - 1;
    const int PI[2] = {pi0, pi1}, PJ[2] = {pj0, pj1};
    float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        if (PI[u] < 0 || PI[u] >= nc) continue;
        const float wi = pw(i, PI[u], nc);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (PJ[q] < 0 || PJ[q] >= nc) continue;
            const float w = wi * pw(j, PJ[q], nc);
            const int64_t C = (int64_t)PI[u] * nc + PJ[q];
#pragma unroll
            for (int f = 0; f < 3; ++f) acc[f] += w * __ldg(e + f * Nc + C);
        }
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) x[f * N + c] += acc[f];
}

// Dense FP64 matrix of a (coarsest) 25-point level: M[(f, c), (g, c + d)].
__global__ void __launch_bounds__(MT) dense_kernel(int n, const float* __restrict__ A,
                                                   double* __restrict__ M) {
    const int64_t N = (int64_t)n * n, K = 3 * N;
    const int64_t t = (int64_t)blockIdx.x * MT + threadIdx.x;
    if (t >= K * K) return;
    const int64_t row = t / K, col = t % K;
    const int f = (int)(row / N), g = (int)(col / N);
    const int64_t c = row % N, c2 = col % N;
    const int di = (int)(c2 / n) - (int)(c / n), dj = (int)(c2 % n) - (int)(c % n);
    double v = 0.0;
    if (di >= -2 && di <= 2 && dj >= -2 && dj <= 2)
        v = (double)A[((int64_t)(3 * f + g) * 25 + (di + 2) * 5 + (dj + 2)) * N + c];
    M[t] = v;
}

// In-place inverse of the symmetric positive (semi)definite K x K matrix M by
// Gauss-Jordan without pivoting, one block.  A pivot at or below 1e-13 of
// the largest diagonal entry marks a null direction: its row and column are
// zeroed (that direction is left out of the solve) instead of dividing.
__global__ void __launch_bounds__(1024) gauss_jordan_kernel(int K, double* __restrict__ M) {
    __shared__ double colk[1024];
    __shared__ double dmax;
    __shared__ int skip;
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int k = 0; k < K; ++k) m = fmax(m, fabs(M[(int64_t)k * K + k]));
        dmax = m;
    }
    __syncthreads();
    for (int k = 0; k < K; ++k) {
        if (threadIdx.x == 0) skip = !(M[(int64_t)k * K + k] > 1e-13 * dmax);
        __syncthreads();
        if (skip) {
            for (int i = threadIdx.x; i < K; i += blockDim.x) {
                M[(int64_t)k * K + i] = 0.0;
                M[(int64_t)i * K + k] = 0.0;
            }
            __syncthreads();
            continue;
        }
        const double piv = 1.0 / M[(int64_t)k * K + k];
        for (int i = threadIdx.x; i < K; i += blockDim.x) colk[i] = M[(int64_t)i * K + k];
        __syncthreads();
        // row k: M[k][j] *= piv, M[k][k] = piv
        for (int j = threadIdx.x; j < K; j += blockDim.x)
            M[(int64_t)k * K + j] = (j == k) ? piv : M[(int64_t)k * K + j] * piv;
        __syncthreads();
        // other rows: M[i][j] -= colk[i] M[k][j]; M[i][k] = -colk[i] piv
        for (int64_t t = threadIdx.x; t < (int64_t)K * K; t += blockDim.x) {
            const int i = (int)(t / K), j = (int)(t % K);
            if (i == k) continue;
            if (j == k)
                M[t] = -colk[i] * piv;
            else
                M[t] -= colk[i] * M[(int64_t)k * K + j];
        }
        __syncthreads();
    }
}

// x = Minv b (FP64 accumulation, FP32 vectors); one warp per row.
__global__ void __launch_bounds__(MT) dense_apply_kernel(int K, const double* __restrict__ Minv,
                                                         const float* __restrict__ b,
                                                         float* __restrict__ x) {
    const int row = (int)(((int64_t)blockIdx.x * MT + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= K) return;
    double acc = 0.0;
    for (int j = lane; j < K; j += 32) acc += Minv[(int64_t)row * K + j] * (double)__ldg(b + j);
    acc = warp_sum(acc);
    if (lane == 0) x[row] = (float)acc;
}

// PCG step scalars (FP64): sc[0] = <r, z>, sc[1] = alpha, sc[2] = beta.
// phase 0: alpha = sc[0] / dots[0]       (dots[0] = <p, A p>)
// phase 1: beta = dots[0] / sc[0], sc[0] = dots[0]   (dots[0] = <r, z>)
// phase 2: sc[0] = dots[0], beta = 0     (first iteration: p = z)
__global__ void pcg_scalars_kernel(const double* __restrict__ dots, double* __restrict__ sc,
                                   int phase) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (phase == 0) {
        const double a = sc[0] / dots[0];
        sc[1] = isfinite(a) ? a : 0.0;
    } else if (phase == 1) {
        const double b = dots[0] / sc[0];
        sc[2] = isfinite(b) ? b : 0.0;
        sc[0] = dots[0];
    } else {
        sc[0] = dots[0];
        sc[2] = 0.0;
    }
}

// x += alpha p; r -= alpha q
__global__ void __launch_bounds__(MT) pcg_xr_kernel(int64_t n, float* __restrict__ x,
                                                    float* __restrict__ r,
                                                    const float* __restrict__ p,
                                                    const float* __restrict__ q,
                                                    const double* __restrict__ sc) {
    const float a = (float)sc[1];
    const int64_t stride = (int64_t)gridDim.x * MT;
    for (int64_t i = (int64_t)blockIdx.x * MT + threadIdx.x; i < n; i += stride) {
        x[i] += a * p[i];
        r[i] -= a * q[i];
    }
}

// p = z + beta p
__global__ void __launch_bounds__(MT) pcg_p_kernel(int64_t n, float* __restrict__ p,
                                                   const float* __restrict__ z,
                                                   const double* __restrict__ sc) {
    const float b = (float)sc[2];
    const int64_t stride = (int64_t)gridDim.x * MT;
    for (int64_t i = (int64_t)blockIdx.x * MT + threadIdx.x; i < n; i += stride)
        p[i] = z[i] + b * p[i];
}

inline unsigned grid_cap(int64_t n) {
    int64_t b = (n + MT - 1) / MT;
    const int64_t cap = 152 * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

bool level_ok(int64_t n) { return n >= 1 && n <= (1 << 15); }

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_nsmg_jx_f32(int64_t n, int32_t neq, const float* coef, const float* x, float* w,
                              void* stream) {
    if (!level_ok(n) || neq < 1 || neq > 16) return ODIL_ERR_SHAPE;
    if (!coef || !x || !w) return ODIL_ERR_ARG;
    jx_kernel<float><<<nblocks(n * n), MT, 0, as_stream(stream)>>>((int)n, neq, coef, x, w);
    return launch_status();
}

ODIL_API int odil_nsmg_jx_f64(int64_t n, int32_t neq, const double* coef, const double* x,
                              double* w, void* stream) {
    if (!level_ok(n) || neq < 1 || neq > 16) return ODIL_ERR_SHAPE;
    if (!coef || !x || !w) return ODIL_ERR_ARG;
    jx_kernel<double><<<nblocks(n * n), MT, 0, as_stream(stream)>>>((int)n, neq, coef, x, w);
    return launch_status();
}

ODIL_API int odil_nsmg_jtw_f32(int64_t n, int32_t neq, const float* coef, const float* w,
                               const float* b, const float* x, const float* dinv, float* out,
                               float omega, int32_t mode, void* stream) {
    if (!level_ok(n) || neq < 1 || neq > 16 || mode < 0 || mode > 2) return ODIL_ERR_SHAPE;
    if (!coef || !w || !out || (mode >= 1 && !b) || (mode == 2 && (!x || !dinv)))
        return ODIL_ERR_ARG;
    jtw_kernel<float><<<nblocks(n * n), MT, 0, as_stream(stream)>>>((int)n, neq, coef, w, b, x,
                                                                    dinv, out, omega, mode);
    return launch_status();
}

ODIL_API int odil_nsmg_jtw_f64(int64_t n, int32_t neq, const double* coef, const double* w,
                               double* out, void* stream) {
    if (!level_ok(n) || neq < 1 || neq > 16) return ODIL_ERR_SHAPE;
    if (!coef || !w || !out) return ODIL_ERR_ARG;
    jtw_kernel<double><<<nblocks(n * n), MT, 0, as_stream(stream)>>>(
        (int)n, neq, coef, w, nullptr, nullptr, nullptr, out, 0.0, 0);
    return launch_status();
}

ODIL_API int odil_nsmg_fine_ata(int64_t n, int32_t neq, const float* coef, float* A,
                                float* dinv, void* stream) {
    if (!level_ok(n) || neq < 1 || neq > 16) return ODIL_ERR_SHAPE;
    if (!coef || !A || !dinv) return ODIL_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    fine_ata_kernel<<<nblocks(9 * n * n), MT, 0, s>>>((int)n, neq, coef, A);
    dinv_kernel<<<nblocks(n * n), MT, 0, s>>>((int)n, A, dinv);
    return launch_status();
}

ODIL_API int odil_nsmg_galerkin(int64_t n, const float* A, float* Ac, float* dinv_c,
                                void* stream) {
    if (!level_ok(n) || n % 2 || n < 2) return ODIL_ERR_SHAPE;
    if (!A || !Ac || !dinv_c) return ODIL_ERR_ARG;
    const int64_t nc = n / 2;
    cudaStream_t s = as_stream(stream);
    galerkin_kernel<<<nblocks(9 * nc * nc), MT, 0, s>>>((int)n, A, Ac);
    dinv_kernel<<<nblocks(nc * nc), MT, 0, s>>>((int)nc, Ac, dinv_c);
    return launch_status();
}

ODIL_API int odil_nsmg_smooth(int64_t n, const float* A, const float* dinv, const float* x,
                              const float* b, float* out, float omega, int32_t mode,
                              void* stream) {
    if (!level_ok(n) || mode < 0 || mode > 2) return ODIL_ERR_SHAPE;
    if (!A || !x || !out || (mode >= 1 && !b) || (mode == 2 && !dinv)) return ODIL_ERR_ARG;
    smooth_kernel<<<nblocks(n * n), MT, 0, as_stream(stream)>>>((int)n, A, dinv, x, b, out,
                                                                omega, mode);
    return launch_status();
}

ODIL_API int odil_nsmg_jacobi0(int64_t n, const float* dinv, const float* b, float* out,
                               float omega, void* stream) {
    if (!level_ok(n)) return ODIL_ERR_SHAPE;
    if (!dinv || !b || !out) return ODIL_ERR_ARG;
    jacobi0_kernel<<<nblocks(n * n), MT, 0, as_stream(stream)>>>(n * n, dinv, b, out, omega);
    return launch_status();
}

ODIL_API int odil_nsmg_restrict(int64_t n, const float* r, float* rc, void* stream) {
    if (!level_ok(n) || n % 2 || n < 2) return ODIL_ERR_SHAPE;
    if (!r || !rc) return ODIL_ERR_ARG;
    restrict_kernel<<<nblocks((n / 2) * (n / 2)), MT, 0, as_stream(stream)>>>((int)n, r, rc);
    return launch_status();
}

ODIL_API int odil_nsmg_prolong_add(int64_t n, const float* e, float* x, void* stream) {
    if (!level_ok(n) || n % 2 || n < 2) return ODIL_ERR_SHAPE;
    if (!e || !x) return ODIL_ERR_ARG;
    prolong_add_kernel<<<nblocks(n * n), MT, 0, as_stream(stream)>>>((int)n, e, x);
    return launch_status();
}

ODIL_API int odil_nsmg_coarse_inverse(int64_t n, const float* A, double* minv, void* stream) {
    const int64_t K = 3 * n * n;
    if (n < 1 || K > 1024) return ODIL_ERR_SHAPE;
    if (!A || !minv) return ODIL_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    dense_kernel<<<nblocks(K * K), MT, 0, s>>>((int)n, A, minv);
    gauss_jordan_kernel<<<1, 1024, 0, s>>>((int)K, minv);
    return launch_status();
}

ODIL_API int odil_nsmg_coarse_apply(int64_t n, const double* minv, const float* b, float* x,
                                    void* stream) {
    const int64_t K = 3 * n * n;
    if (n < 1 || K > 1024) return ODIL_ERR_SHAPE;
    if (!minv || !b || !x) return ODIL_ERR_ARG;
    dense_apply_kernel<<<nblocks(K * 32), MT, 0, as_stream(stream)>>>((int)K, minv, b, x);
    return launch_status();
}

ODIL_API int odil_pcg_scalars(const double* dots, double* sc, int32_t phase, void* stream) {
    if (!dots || !sc || phase < 0 || phase > 2) return ODIL_ERR_ARG;
    pcg_scalars_kernel<<<1, 32, 0, as_stream(stream)>>>(dots, sc, phase);
    return launch_status();
}

ODIL_API int odil_pcg_update_xr(int64_t n, float* x, float* r, const float* p, const float* q,
                                const double* sc, void* stream) {
    if (n < 1) return ODIL_ERR_SHAPE;
    if (!x || !r || !p || !q || !sc) return ODIL_ERR_ARG;
    pcg_xr_kernel<<<grid_cap(n), MT, 0, as_stream(stream)>>>(n, x, r, p, q, sc);
    return launch_status();
}

ODIL_API int odil_pcg_update_p(int64_t n, float* p, const float* z, const double* sc,
                               void* stream) {
    if (n < 1) return ODIL_ERR_SHAPE;
    if (!p || !z || !sc) return ODIL_ERR_ARG;
    pcg_p_kernel<<<grid_cap(n), MT, 0, as_stream(stream)>>>(n, p, z, sc);
    return launch_status();
}
