// Multigrid decomposition kernels (multigrid.py:1217-1426): one level of
// refinement per launch, fused with the scale and the add of the level's own
// weights (weights_to_field), and its adjoint, fused with the scaled copies
// that make the weights' gradient.  One thread per output point; the
// per-point arithmetic is in mgdecomp.cuh.
#include "common.cuh"
#include "mgdecomp.cuh"

namespace odil {
namespace {

using mgd::Grid;

constexpr int kThreads = 256;

// DIM and CELL are fixed per instantiation so that the per-axis loops of
// mgdecomp.cuh unroll and their small arrays stay in registers.  ROWS: the
// launch grid is the index grid itself (x: the last axis in blocks of
// kThreads, y and z: the other axes, each at most 65535), so a thread finds
// its point without the 64-bit divisions of unflatten; otherwise a
// grid-stride loop over the flat index.
template <int DIM, bool ROWS>
__device__ __forceinline__ bool row_index(const int64_t* size, int64_t* o, int64_t* i) {
    const int64_t last = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (last >= size[DIM - 1]) return false;
    o[0] = o[1] = o[2] = 0;
    o[DIM - 1] = last;
    if (DIM >= 2) o[DIM - 2] = blockIdx.y;
    if (DIM == 3) o[0] = blockIdx.z;
    *i = (o[0] * size[1] + o[1]) * size[2] + o[2];
    return true;
}

template <typename T, int DIM, int CELL, bool ROWS>
__global__ void __launch_bounds__(kThreads)
    mgd_refine_kernel(Grid g, const T* __restrict__ in, T* __restrict__ out, T alpha,
                      const T* __restrict__ add, T beta, int64_t total) {
    g.dim = DIM;
    g.cell = CELL;
    if constexpr (ROWS) {
        int64_t o[3], i;
        if (!row_index<DIM, ROWS>(g.m, o, &i)) return;
        T v = alpha * mgd::refine_point(g, in, o);
        if (add) v += beta * add[i];
        out[i] = v;
    } else {
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
             i += (int64_t)gridDim.x * blockDim.x) {
            int64_t o[3] = {0, 0, 0};
            mgd::unflatten(g.m, g.dim, i, o);
            T v = alpha * mgd::refine_point(g, in, o);
            if (add) v += beta * add[i];
            out[i] = v;
        }
    }
}

template <typename T, int DIM, int CELL, bool ROWS>
__global__ void __launch_bounds__(kThreads)
    mgd_refine_t_kernel(Grid g, const T* __restrict__ gf, T* __restrict__ gc,
                        T* __restrict__ wc, T alpha_c, T* __restrict__ wf, T beta_f,
                        int64_t total) {
    g.dim = DIM;
    g.cell = CELL;
    if constexpr (ROWS) {
        int64_t q[3], i;
        if (!row_index<DIM, ROWS>(g.n, q, &i)) return;
        const T v = mgd::refine_adjoint_point(g, gf, q);
        if (gc) gc[i] = v;
        if (wc) wc[i] = alpha_c * v;
        if (wf) mgd::scale_owned(g, gf, wf, beta_f, q);
    } else {
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
             i += (int64_t)gridDim.x * blockDim.x) {
            int64_t q[3] = {0, 0, 0};
            mgd::unflatten(g.n, g.dim, i, q);
            const T v = mgd::refine_adjoint_point(g, gf, q);
            if (gc) gc[i] = v;
            if (wc) wc[i] = alpha_c * v;
            if (wf) mgd::scale_owned(g, gf, wf, beta_f, q);
        }
    }
}

// The row grid of an index grid `size` of `dim` axes, if it fits.
bool row_grid(const int64_t* size, int dim, dim3* grid) {
    const int64_t bx = (size[dim - 1] + kThreads - 1) / kThreads;
    const int64_t by = dim >= 2 ? size[dim - 2] : 1;
    const int64_t bz = dim == 3 ? size[0] : 1;
    if (bx > 0x7fffffff || by > 65535 || bz > 65535) return false;
    *grid = dim3((unsigned)bx, (unsigned)by, (unsigned)bz);
    return true;
}

int make_grid(int32_t dim, const int64_t* n, int32_t cell, Grid* g) {
    if (dim < 1 || dim > 3 || !n || (cell != 0 && cell != 1)) return ODIL_ERR_ARG;
    g->dim = dim;
    g->cell = cell;
    for (int d = 0; d < 3; ++d) {
        g->n[d] = 1;
        g->m[d] = 1;
    }
    for (int d = 0; d < dim; ++d) {
        // Cell refinement extrapolates from two cells per axis.
        if (n[d] < (cell ? 2 : 1) || n[d] > (int64_t(1) << 40)) return ODIL_ERR_SHAPE;
        g->n[d] = n[d];
        g->m[d] = mgd::fine_size(n[d], cell);
    }
    return ODIL_OK;
}

int grid_blocks(int64_t total) {
    int64_t b = (total + kThreads - 1) / kThreads;
    const int64_t cap = 152 * 16;  // SMs x resident blocks; the loop strides past it
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <typename T>
int refine_impl(int32_t dim, const int64_t* n, int32_t cell, const T* in, T* out, double alpha,
                const T* add, double beta, void* stream) {
    Grid g;
    int st = make_grid(dim, n, cell, &g);
    if (st) return st;
    if (!in || !out) return ODIL_ERR_ARG;
    const int64_t total = g.m[0] * g.m[1] * g.m[2];
    dim3 rg;
    const bool rows = row_grid(g.m, dim, &rg);
    decltype(&mgd_refine_kernel<T, 1, 0, true>) kern;
#define ODIL_MGD_PICK(R)                                                  \
    switch (dim * 2 + cell) {                                             \
        case 2: kern = mgd_refine_kernel<T, 1, 0, R>; break;              \
        case 3: kern = mgd_refine_kernel<T, 1, 1, R>; break;              \
        case 4: kern = mgd_refine_kernel<T, 2, 0, R>; break;              \
        case 5: kern = mgd_refine_kernel<T, 2, 1, R>; break;              \
        case 6: kern = mgd_refine_kernel<T, 3, 0, R>; break;              \
        default: kern = mgd_refine_kernel<T, 3, 1, R>; break;             \
    }
    if (rows) {
        ODIL_MGD_PICK(true)
    } else {
        ODIL_MGD_PICK(false)
    }
#undef ODIL_MGD_PICK
    const dim3 grid = rows ? rg : dim3((unsigned)grid_blocks(total));
    kern<<<grid, kThreads, 0, as_stream(stream)>>>(g, in, out, (T)alpha, add, (T)beta, total);
    return launch_status();
}

template <typename T>
int refine_t_impl(int32_t dim, const int64_t* n, int32_t cell, const T* gf, T* gc, T* wc,
                  double alpha_c, T* wf, double beta_f, void* stream) {
    Grid g;
    int st = make_grid(dim, n, cell, &g);
    if (st) return st;
    if (!gf || (!gc && !wc && !wf)) return ODIL_ERR_ARG;
    const int64_t total = g.n[0] * g.n[1] * g.n[2];
    dim3 rg;
    const bool rows = row_grid(g.n, dim, &rg);
    decltype(&mgd_refine_t_kernel<T, 1, 0, true>) kern;
#define ODIL_MGD_PICK(R)                                                  \
    switch (dim * 2 + cell) {                                             \
        case 2: kern = mgd_refine_t_kernel<T, 1, 0, R>; break;            \
        case 3: kern = mgd_refine_t_kernel<T, 1, 1, R>; break;            \
        case 4: kern = mgd_refine_t_kernel<T, 2, 0, R>; break;            \
        case 5: kern = mgd_refine_t_kernel<T, 2, 1, R>; break;            \
        case 6: kern = mgd_refine_t_kernel<T, 3, 0, R>; break;            \
        default: kern = mgd_refine_t_kernel<T, 3, 1, R>; break;           \
    }
    if (rows) {
        ODIL_MGD_PICK(true)
    } else {
        ODIL_MGD_PICK(false)
    }
#undef ODIL_MGD_PICK
    const dim3 grid = rows ? rg : dim3((unsigned)grid_blocks(total));
    kern<<<grid, kThreads, 0, as_stream(stream)>>>(g, gf, gc, wc, (T)alpha_c, wf, (T)beta_f,
                                                   total);
    return launch_status();
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_mgdecomp_refine_f32(int32_t dim, const int64_t* n, int32_t cell,
                                      const float* in, float* out, double alpha,
                                      const float* add, double beta, void* stream) {
    return refine_impl<float>(dim, n, cell, in, out, alpha, add, beta, stream);
}
ODIL_API int odil_mgdecomp_refine_f64(int32_t dim, const int64_t* n, int32_t cell,
                                      const double* in, double* out, double alpha,
                                      const double* add, double beta, void* stream) {
    return refine_impl<double>(dim, n, cell, in, out, alpha, add, beta, stream);
}
ODIL_API int odil_mgdecomp_refine_t_f32(int32_t dim, const int64_t* n, int32_t cell,
                                        const float* g, float* gc, float* wc, double alpha_c,
                                        float* wf, double beta_f, void* stream) {
    return refine_t_impl<float>(dim, n, cell, g, gc, wc, alpha_c, wf, beta_f, stream);
}
ODIL_API int odil_mgdecomp_refine_t_f64(int32_t dim, const int64_t* n, int32_t cell,
                                        const double* g, double* gc, double* wc,
                                        double alpha_c, double* wf, double beta_f,
                                        void* stream) {
    return refine_t_impl<double>(dim, n, cell, g, gc, wc, alpha_c, wf, beta_f, stream);
}
