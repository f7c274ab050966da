// Direct solve of the Newton system of the cavity (3 equations u, v, p on an
// n x n grid) with the pressure pinned at one cell, in FP32 for iterative
// refinement in FP64 by the caller.
//
// Reference: linsolver.py:28-45 solves the normal equations J^T J d = -J^T f
// with SuperLU.  For the forward problem J is square; its pressure is
// determined up to a constant, and the continuity residuals sum to the
// boundary flux, so one continuity equation is redundant.  Replacing the
// continuity row of the pinned cell by "p[pin] = 0" gives a nonsingular square
// system with the same solution as the least-squares one (up to the constant
// the reference leaves free), solved here directly.
//
// The Jacobian couples a cell to its four neighbours only (shifts of
// stencil_var, ns_steady.py), so ordered by grid rows k (the first array axis)
// it is block tridiagonal with blocks of m = 3n unknowns (f, j) -> f n + j:
//   L_k d_{k-1} + D_k d_k + U_k d_{k+1} = b_k,
// D_k banded (neighbours j -+ 1), L_k and U_k diagonal per (equation, field).
// Block LU (block Thomas): S_0 = D_0, S_k = D_k - L_k W_{k-1}, W_k = S_k^-1 U_k.
// Each S_k is factored by cuSOLVER's dense LU with partial pivoting (a library
// dense factorisation, like a library GEMM) and inverted explicitly (LU solve
// against the identity), so that W_k = S_k^-1 U_k is a 3-column combination
// per column (U_k is diagonal per (equation, field)) and every later solve is
// two memory-bound GEMVs per block row instead of triangular solves:
// y_k = S_k^-1 (b_k - L_k y_{k-1}), then x_k = y_k - W_k x_{k+1}.  Storage:
// n m^2 floats for the inverses, (n-1) m^2 for W and m^2 of scratch: 9.7 GB
// at n = 512.
//
// cuSOLVER and cuBLAS handles are created once per device on first use (their
// own allocations); make that first call before any stream capture.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <vector>

#include "common.cuh"

namespace odil {
namespace {

constexpr int kMaxDev = 64;
cusolverDnHandle_t g_sol[kMaxDev];
cublasHandle_t g_blas[kMaxDev];

int handles(cudaStream_t s, cusolverDnHandle_t* sol, cublasHandle_t* blas) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return ODIL_ERR_LAUNCH;
    if (!g_sol[dev] && cusolverDnCreate(&g_sol[dev]) != CUSOLVER_STATUS_SUCCESS) {
        g_sol[dev] = nullptr;
        return ODIL_ERR_LAUNCH;
    }
    if (!g_blas[dev] && cublasCreate(&g_blas[dev]) != CUBLAS_STATUS_SUCCESS) {
        g_blas[dev] = nullptr;
        return ODIL_ERR_LAUNCH;
    }
    if (cusolverDnSetStream(g_sol[dev], s) != CUSOLVER_STATUS_SUCCESS) return ODIL_ERR_LAUNCH;
    if (cublasSetStream(g_blas[dev], s) != CUBLAS_STATUS_SUCCESS) return ODIL_ERR_LAUNCH;
    *sol = g_sol[dev];
    *blas = g_blas[dev];
    return ODIL_OK;
}

// Workspace layout, each part 256-byte aligned.
struct NdLayout {
    int64_t n, m;
    int64_t off_lu, off_w, off_s, off_piv, off_info, off_y, off_t, off_work, total;
};

inline int64_t al256(int64_t b) { return (b + 255) / 256 * 256; }

NdLayout nd_layout(int64_t n, int64_t lwork) {
    NdLayout q;
    q.n = n;
    q.m = 3 * n;
    const int64_t mm = q.m * q.m * (int64_t)sizeof(float);
    int64_t o = 0;
    q.off_lu = o;   o += al256(n * mm);  // S_k^-1 per block row
    q.off_w = o;    o += al256((n > 1 ? n - 1 : 1) * mm);
    q.off_s = o;    o += al256(mm);      // LU scratch
    q.off_piv = o;  o += al256(n * q.m * (int64_t)sizeof(int));
    q.off_info = o; o += al256((n + 1) * (int64_t)sizeof(int));  // getrf per block + getrs
    q.off_y = o;    o += al256(n * q.m * (int64_t)sizeof(float));
    q.off_t = o;    o += al256(q.m * (int64_t)sizeof(float));
    q.off_work = o; o += al256(lwork * (int64_t)sizeof(float));
    q.total = o;
    return q;
}

// Coefficient of equation e, field f, stencil slot s at cell (k, j); the
// pinned row (equation 2 at the pinned cell) is the identity on p there.
__device__ __forceinline__ float cf(const double* __restrict__ coef, int64_t N, int n, int e,
                                    int f, int s, int k, int j) {
    return (float)__ldg(coef + ((int64_t)(e * 15 + f * 5 + s)) * N + (int64_t)k * n + j);
}

// D_k (column-major m x m, zeroed before): the in-row stencil (shifts (0,0),
// (0,-1), (0,+1); slots 0, 3, 4).
__global__ void nd_fill_diag(const double* __restrict__ coef, int n, int k, int pin_k,
                             int pin_j, float* __restrict__ D) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;  // row (e, j)
    const int m = 3 * n;
    if (r >= m) return;
    const int e = r / n, j = r - e * n;
    const int64_t N = (int64_t)n * n;
    if (e == 2 && k == pin_k && j == pin_j) {
        D[r + (int64_t)r * m] = 1.f;
        return;
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        D[r + (int64_t)(f * n + j) * m] = cf(coef, N, n, e, f, 0, k, j);
        if (j > 0) D[r + (int64_t)(f * n + j - 1) * m] = cf(coef, N, n, e, f, 3, k, j);
        if (j + 1 < n) D[r + (int64_t)(f * n + j + 1) * m] = cf(coef, N, n, e, f, 4, k, j);
    }
}

// W_k = S_k^-1 U_k with U_k[(e, j), (f, j)] = coefficient of equation e,
// field f, shift (+1, 0) (slot 2) at cell (k, j); the pinned row of U_k is 0.
// Column (f, j) of W is sum_e U[(e, j), (f, j)] * column (e, j) of S_k^-1.
__global__ void nd_w_from_inverse(const double* __restrict__ coef, int n, int k, int pin_k,
                                  int pin_j, const float* __restrict__ Sinv,
                                  float* __restrict__ W) {
    const int m = 3 * n;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;  // row of W
    if (r >= m) return;
    const int64_t N = (int64_t)n * n;
    for (int c = blockIdx.y; c < m; c += gridDim.y) {  // column (f, j)
        const int f = c / n, j = c - f * n;
        float acc = 0.f;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            if (e == 2 && k == pin_k && j == pin_j) continue;
            acc = fmaf(Sinv[r + (int64_t)(e * n + j) * m], cf(coef, N, n, e, f, 2, k, j), acc);
        }
        W[r + (int64_t)c * m] = acc;
    }
}

// Identity (column-major m x m, zeroed before).
__global__ void nd_identity(int m, float* __restrict__ A) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < m) A[r + (int64_t)r * m] = 1.f;
}

// S_k = D_k - L_k W_{k-1}; L_k: shift (-1, 0), slot 1.  Thread per element,
// consecutive threads down a column (coalesced in column-major storage).
__global__ void nd_schur(const double* __restrict__ coef, int n, int k, int pin_k, int pin_j,
                         const float* __restrict__ W, float* __restrict__ D) {
    const int m = 3 * n;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int e = r / n, j = r - e * n;
    if (e == 2 && k == pin_k && j == pin_j) return;
    const int64_t N = (int64_t)n * n;
    const float l0 = cf(coef, N, n, e, 0, 1, k, j);
    const float l1 = cf(coef, N, n, e, 1, 1, k, j);
    const float l2 = cf(coef, N, n, e, 2, 1, k, j);
    for (int c = blockIdx.y; c < m; c += gridDim.y) {
        const float* w = W + (int64_t)c * m + j;
        float acc = l0 * w[0];
        acc = fmaf(l1, w[n], acc);
        acc = fmaf(l2, w[2 * n], acc);
        D[r + (int64_t)c * m] -= acc;
    }
}

// t = b_k - L_k y_{k-1} (b field-major FP32; y block-major).
__global__ void nd_rhs(const double* __restrict__ coef, int n, int k, int pin_k, int pin_j,
                       const float* __restrict__ b, const float* __restrict__ yprev,
                       float* __restrict__ t) {
    const int m = 3 * n;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int e = r / n, j = r - e * n;
    const int64_t N = (int64_t)n * n;
    float v = b[(int64_t)e * N + (int64_t)k * n + j];
    if (yprev && !(e == 2 && k == pin_k && j == pin_j)) {
        v -= cf(coef, N, n, e, 0, 1, k, j) * yprev[j];
        v -= cf(coef, N, n, e, 1, 1, k, j) * yprev[n + j];
        v -= cf(coef, N, n, e, 2, 1, k, j) * yprev[2 * n + j];
    }
    t[r] = v;
}

// x (field-major) from y (block-major).
__global__ void nd_scatter(int n, const float* __restrict__ y, float* __restrict__ x) {
    const int64_t N = (int64_t)n * n;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * N) return;
    const int64_t k = i / (3 * n);
    const int r = (int)(i - k * 3 * n);
    const int f = r / n, j = r - f * n;
    x[(int64_t)f * N + k * n + j] = y[i];
}

// y (block-major) from b (field-major).
__global__ void nd_gather(int n, const float* __restrict__ b, float* __restrict__ y) {
    const int64_t N = (int64_t)n * n;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * N) return;
    const int64_t k = i / (3 * n);
    const int r = (int)(i - k * 3 * n);
    const int f = r / n, j = r - f * n;
    y[i] = b[(int64_t)f * N + k * n + j];
}

// t = y_k - L_{k+1}^T x_{k+1}: (L^T x)[(f, j)] = sum_e L[(e, j), (f, j)] x[(e, j)]
// with L_{k+1}[(e, j), (f, j)] the slot-1 coefficient at cell (k+1, j) (zero
// on the pinned row).
__global__ void nd_rhs_t(const double* __restrict__ coef, int n, int k1, int pin_k, int pin_j,
                         const float* __restrict__ yk, const float* __restrict__ x1,
                         float* __restrict__ t) {
    const int m = 3 * n;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int f = r / n, j = r - f * n;
    const int64_t N = (int64_t)n * n;
    float v = yk[r];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        if (e == 2 && k1 == pin_k && j == pin_j) continue;
        v -= cf(coef, N, n, e, f, 1, k1, j) * x1[e * n + j];
    }
    t[r] = v;
}

int check(int64_t n, int64_t pin) {
    if (n < 2 || n > 4096) return ODIL_ERR_SHAPE;
    if (pin < 0 || pin >= n * n) return ODIL_ERR_ARG;
    return ODIL_OK;
}

int lwork_of(int64_t n, int64_t* lwork) {
    cusolverDnHandle_t sol;
    cublasHandle_t blas;
    int st = handles(nullptr, &sol, &blas);
    if (st) return st;
    const int m = (int)(3 * n);
    int lw = 0;
    if (cusolverDnSgetrf_bufferSize(sol, m, m, nullptr, m, &lw) != CUSOLVER_STATUS_SUCCESS)
        return ODIL_ERR_LAUNCH;
    *lwork = lw;
    return ODIL_OK;
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int64_t odil_ns_direct_workspace_bytes(int64_t n) {
    if (n < 2 || n > 4096) return -1;
    int64_t lwork = 0;
    if (lwork_of(n, &lwork)) return -1;
    return nd_layout(n, lwork).total;
}

ODIL_API int odil_ns_direct_factor(int64_t n, const double* coef, int64_t pin, void* ws,
                                   int64_t ws_bytes, void* stream) {
    int st = check(n, pin);
    if (st) return st;
    if (!coef || !ws) return ODIL_ERR_ARG;
    int64_t lwork = 0;
    if ((st = lwork_of(n, &lwork))) return st;
    const NdLayout q = nd_layout(n, lwork);
    if (ws_bytes < q.total) return ODIL_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    cusolverDnHandle_t sol;
    cublasHandle_t blas;
    if ((st = handles(s, &sol, &blas))) return st;
    char* base = reinterpret_cast<char*>(ws);
    float* INV = reinterpret_cast<float*>(base + q.off_lu);
    float* W = reinterpret_cast<float*>(base + q.off_w);
    int* piv = reinterpret_cast<int*>(base + q.off_piv);
    int* info = reinterpret_cast<int*>(base + q.off_info);
    float* work = reinterpret_cast<float*>(base + q.off_work);
    const int m = (int)q.m, nn = (int)n;
    const int pk = (int)(pin / n), pj = (int)(pin % n);
    const int64_t mm = (int64_t)m * m;
    const int tb = 128, rb = (m + tb - 1) / tb;
    float* S = reinterpret_cast<float*>(base + q.off_s);
    for (int k = 0; k < nn; ++k) {
        float* Inv = INV + k * mm;
        if (cudaMemsetAsync(S, 0, mm * sizeof(float), s) != cudaSuccess) return ODIL_ERR_LAUNCH;
        nd_fill_diag<<<rb, tb, 0, s>>>(coef, nn, k, pk, pj, S);
        if (k > 0) {
            nd_schur<<<dim3(rb, 256), tb, 0, s>>>(coef, nn, k, pk, pj, W + (k - 1) * mm, S);
        }
        if (cusolverDnSgetrf(sol, m, m, S, m, work, piv + (int64_t)k * m, info + k) !=
            CUSOLVER_STATUS_SUCCESS)
            return ODIL_ERR_LAUNCH;
        if (cudaMemsetAsync(Inv, 0, mm * sizeof(float), s) != cudaSuccess) return ODIL_ERR_LAUNCH;
        nd_identity<<<rb, tb, 0, s>>>(m, Inv);
        if (cusolverDnSgetrs(sol, CUBLAS_OP_N, m, m, S, m, piv + (int64_t)k * m, Inv, m,
                             info + n) != CUSOLVER_STATUS_SUCCESS)
            return ODIL_ERR_LAUNCH;
        if (k + 1 < nn) {
            nd_w_from_inverse<<<dim3(rb, 256), tb, 0, s>>>(coef, nn, k, pk, pj, Inv, W + k * mm);
        }
    }
    return launch_status();
}

// Singular pivots of the last factorisation: the number of blocks whose
// getrf info is nonzero (0 = every factor nonsingular).  Synchronises the
// stream.
ODIL_API int odil_ns_direct_check(int64_t n, const void* ws, void* stream) {
    if (n < 2 || n > 4096 || !ws) return ODIL_ERR_ARG;
    int64_t lwork = 0;
    int st = lwork_of(n, &lwork);
    if (st) return st;
    const NdLayout q = nd_layout(n, lwork);
    const int* info = reinterpret_cast<const int*>(reinterpret_cast<const char*>(ws) + q.off_info);
    std::vector<int> h((size_t)n);
    cudaStream_t s = as_stream(stream);
    if (cudaMemcpyAsync(h.data(), info, n * sizeof(int), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return ODIL_ERR_LAUNCH;
    int bad = 0;
    for (int v : h) bad += v != 0;
    return bad;
}

ODIL_API int odil_ns_direct_solve(int64_t n, const double* coef, int64_t pin, void* ws,
                                  int64_t ws_bytes, const float* b, float* x, void* stream) {
    int st = check(n, pin);
    if (st) return st;
    if (!coef || !ws || !b || !x) return ODIL_ERR_ARG;
    int64_t lwork = 0;
    if ((st = lwork_of(n, &lwork))) return st;
    const NdLayout q = nd_layout(n, lwork);
    if (ws_bytes < q.total) return ODIL_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    cusolverDnHandle_t sol;
    cublasHandle_t blas;
    if ((st = handles(s, &sol, &blas))) return st;
    char* base = reinterpret_cast<char*>(ws);
    const float* INV = reinterpret_cast<const float*>(base + q.off_lu);  // S_k^-1
    const float* W = reinterpret_cast<const float*>(base + q.off_w);
    float* y = reinterpret_cast<float*>(base + q.off_y);
    const int m = (int)q.m, nn = (int)n;
    const int pk = (int)(pin / n), pj = (int)(pin % n);
    const int64_t mm = (int64_t)m * m;
    const int tb = 128, rb = (m + tb - 1) / tb;
    float* t = reinterpret_cast<float*>(base + q.off_t);
    const float minus1 = -1.f, one = 1.f, zero = 0.f;
    if (cublasSetPointerMode(blas, CUBLAS_POINTER_MODE_HOST) != CUBLAS_STATUS_SUCCESS)
        return ODIL_ERR_LAUNCH;
    for (int k = 0; k < nn; ++k) {
        float* yk = y + (int64_t)k * m;
        nd_rhs<<<rb, tb, 0, s>>>(coef, nn, k, pk, pj, b, k > 0 ? yk - m : nullptr, t);
        if (cublasSgemv(blas, CUBLAS_OP_N, m, m, &one, INV + k * mm, m, t, 1, &zero, yk, 1) !=
            CUBLAS_STATUS_SUCCESS)
            return ODIL_ERR_LAUNCH;
    }
    for (int k = nn - 2; k >= 0; --k) {
        if (cublasSgemv(blas, CUBLAS_OP_N, m, m, &minus1, W + k * mm, m, y + (int64_t)(k + 1) * m,
                        1, &one, y + (int64_t)k * m, 1) != CUBLAS_STATUS_SUCCESS)
            return ODIL_ERR_LAUNCH;
    }
    const int64_t tot = 3 * (int64_t)n * n;
    nd_scatter<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(nn, y, x);
    return launch_status();
}

// Transposed solve J'^T x = b with the same factors: J' = Lt Ut with Lt block
// lower bidiagonal (diagonal S_k, subdiagonal L_k) and Ut block upper
// bidiagonal (identity diagonal, superdiagonal W_k = S_k^-1 U_k), so
// Ut^T y = b:  y_k = b_k - W_{k-1}^T y_{k-1};
// Lt^T x = y:  x_k = S_k^-T (y_k - L_{k+1}^T x_{k+1}).
// Transposed GEMVs on the stored S_k^-1 and W_k.
ODIL_API int odil_ns_direct_solve_t(int64_t n, const double* coef, int64_t pin, void* ws,
                                    int64_t ws_bytes, const float* b, float* x, void* stream) {
    int st = check(n, pin);
    if (st) return st;
    if (!coef || !ws || !b || !x) return ODIL_ERR_ARG;
    int64_t lwork = 0;
    if ((st = lwork_of(n, &lwork))) return st;
    const NdLayout q = nd_layout(n, lwork);
    if (ws_bytes < q.total) return ODIL_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    cusolverDnHandle_t sol;
    cublasHandle_t blas;
    if ((st = handles(s, &sol, &blas))) return st;
    char* base = reinterpret_cast<char*>(ws);
    const float* INV = reinterpret_cast<const float*>(base + q.off_lu);
    const float* W = reinterpret_cast<const float*>(base + q.off_w);
    float* y = reinterpret_cast<float*>(base + q.off_y);
    float* t = reinterpret_cast<float*>(base + q.off_t);
    const int m = (int)q.m, nn = (int)n;
    const int pk = (int)(pin / n), pj = (int)(pin % n);
    const int64_t mm = (int64_t)m * m;
    const int tb = 128, rb = (m + tb - 1) / tb;
    const float minus1 = -1.f, one = 1.f, zero = 0.f;
    if (cublasSetPointerMode(blas, CUBLAS_POINTER_MODE_HOST) != CUBLAS_STATUS_SUCCESS)
        return ODIL_ERR_LAUNCH;
    const int64_t tot = 3 * (int64_t)n * n;
    nd_gather<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(nn, b, y);
    for (int k = 1; k < nn; ++k) {
        if (cublasSgemv(blas, CUBLAS_OP_T, m, m, &minus1, W + (k - 1) * mm, m,
                        y + (int64_t)(k - 1) * m, 1, &one, y + (int64_t)k * m, 1) !=
            CUBLAS_STATUS_SUCCESS)
            return ODIL_ERR_LAUNCH;
    }
    // x overwrites y block by block from the last one (x_{k+1} is read
    // before block k is overwritten).
    for (int k = nn - 1; k >= 0; --k) {
        float* yk = y + (int64_t)k * m;
        if (k + 1 < nn) {
            nd_rhs_t<<<rb, tb, 0, s>>>(coef, nn, k + 1, pk, pj, yk, yk + m, t);
        } else if (cudaMemcpyAsync(t, yk, m * sizeof(float), cudaMemcpyDeviceToDevice, s) !=
                   cudaSuccess) {
            return ODIL_ERR_LAUNCH;
        }
        if (cublasSgemv(blas, CUBLAS_OP_T, m, m, &one, INV + k * mm, m, t, 1, &zero, yk, 1) !=
            CUBLAS_STATUS_SUCCESS)
            return ODIL_ERR_LAUNCH;
    }
    nd_scatter<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(nn, y, x);
    return launch_status();
}

// Explicit inverse of a small dense FP64 matrix (column-major n x n; the
// coarsest multigrid operators, n <= 1024): cuSOLVER LU with partial
// pivoting and a solve against the identity.  Returns ODIL_ERR_NONFINITE when
// a pivot is exactly zero (synchronises the stream to read it).
__global__ void nd_identity64(int n, double* __restrict__ A) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) A[r + (int64_t)r * n] = 1.0;
}

ODIL_API int64_t odil_dense_inverse_workspace_bytes(int64_t n) {
    if (n < 1 || n > 4096) return -1;
    cusolverDnHandle_t sol;
    cublasHandle_t blas;
    if (handles(nullptr, &sol, &blas)) return -1;
    int lw = 0;
    if (cusolverDnDgetrf_bufferSize(sol, (int)n, (int)n, nullptr, (int)n, &lw) !=
        CUSOLVER_STATUS_SUCCESS)
        return -1;
    return al256(n * n * (int64_t)sizeof(double)) + al256(n * (int64_t)sizeof(int)) + 256 +
           al256((int64_t)lw * (int64_t)sizeof(double));
}

ODIL_API int odil_dense_inverse_f64(int64_t n, const double* A, double* Ainv, void* ws,
                                    int64_t ws_bytes, void* stream) {
    if (n < 1 || n > 4096) return ODIL_ERR_SHAPE;
    if (!A || !Ainv || !ws) return ODIL_ERR_ARG;
    const int64_t need = odil_dense_inverse_workspace_bytes(n);
    if (need < 0) return ODIL_ERR_LAUNCH;
    if (ws_bytes < need) return ODIL_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    cusolverDnHandle_t sol;
    cublasHandle_t blas;
    int st = handles(s, &sol, &blas);
    if (st) return st;
    char* base = reinterpret_cast<char*>(ws);
    double* LU = reinterpret_cast<double*>(base);
    int* piv = reinterpret_cast<int*>(base + al256(n * n * (int64_t)sizeof(double)));
    int* info = reinterpret_cast<int*>(reinterpret_cast<char*>(piv) +
                                       al256(n * (int64_t)sizeof(int)));
    double* work = reinterpret_cast<double*>(reinterpret_cast<char*>(info) + 256);
    const int m = (int)n;
    if (cudaMemcpyAsync(LU, A, n * n * sizeof(double), cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess ||
        cudaMemsetAsync(Ainv, 0, n * n * sizeof(double), s) != cudaSuccess)
        return ODIL_ERR_LAUNCH;
    nd_identity64<<<(m + 127) / 128, 128, 0, s>>>(m, Ainv);
    if (cusolverDnDgetrf(sol, m, m, LU, m, work, piv, info) != CUSOLVER_STATUS_SUCCESS)
        return ODIL_ERR_LAUNCH;
    int h = 0;
    if (cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return ODIL_ERR_LAUNCH;
    if (h != 0) return ODIL_ERR_NONFINITE;
    if (cusolverDnDgetrs(sol, CUBLAS_OP_N, m, m, LU, m, piv, Ainv, m, info + 1) !=
        CUSOLVER_STATUS_SUCCESS)
        return ODIL_ERR_LAUNCH;
    return launch_status();
}
