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
// mgdecomp.cuh unroll and their small arrays stay in registers.
template <typename T, int DIM, int CELL>
__global__ void __launch_bounds__(kThreads)
    mgd_refine_kernel(Grid g, const T* __restrict__ in, T* __restrict__ out, T alpha,
                      const T* __restrict__ add, T beta, int64_t total) {
    g.dim = DIM;
    g.cell = CELL;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t o[3] = {0, 0, 0};
        mgd::unflatten(g.m, g.dim, i, o);
        T v = alpha * mgd::refine_point(g, in, o);
        if (add) v += beta * add[i];
        out[i] = v;
    }
}

template <typename T, int DIM, int CELL>
__global__ void __launch_bounds__(kThreads)
    mgd_refine_t_kernel(Grid g, const T* __restrict__ gf, T* __restrict__ gc,
                        T* __restrict__ wc, T alpha_c, T* __restrict__ wf, T beta_f,
                        int64_t total) {
    g.dim = DIM;
    g.cell = CELL;
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
    decltype(&mgd_refine_kernel<T, 1, 0>) kern;
    switch (dim * 2 + cell) {
        case 2: kern = mgd_refine_kernel<T, 1, 0>; break;
        case 3: kern = mgd_refine_kernel<T, 1, 1>; break;
        case 4: kern = mgd_refine_kernel<T, 2, 0>; break;
        case 5: kern = mgd_refine_kernel<T, 2, 1>; break;
        case 6: kern = mgd_refine_kernel<T, 3, 0>; break;
        default: kern = mgd_refine_kernel<T, 3, 1>; break;
    }
    kern<<<grid_blocks(total), kThreads, 0, as_stream(stream)>>>(g, in, out, (T)alpha, add,
                                                                 (T)beta, total);
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
    decltype(&mgd_refine_t_kernel<T, 1, 0>) kern;
    switch (dim * 2 + cell) {
        case 2: kern = mgd_refine_t_kernel<T, 1, 0>; break;
        case 3: kern = mgd_refine_t_kernel<T, 1, 1>; break;
        case 4: kern = mgd_refine_t_kernel<T, 2, 0>; break;
        case 5: kern = mgd_refine_t_kernel<T, 2, 1>; break;
        case 6: kern = mgd_refine_t_kernel<T, 3, 0>; break;
        default: kern = mgd_refine_t_kernel<T, 3, 1>; break;
    }
    kern<<<grid_blocks(total), kThreads, 0, as_stream(stream)>>>(g, gf, gc, wc, (T)alpha_c, wf,
                                                                 (T)beta_f, total);
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
