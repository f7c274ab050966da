// Multigrid decomposition of a field (multigrid.py:1217-1426): one level of
// refinement of a coarse grid and its adjoint, as per-point functions.
//
// Node grids refine n -> 2n - 1: fine node 2i takes u[i], fine node 2i + 1
// the mean of u[i] and u[i + 1], per axis (multilinear interpolation).
// Cell grids refine n -> 2n: fine cell 2k takes 3/4 u[k] + 1/4 u[k - 1], fine
// cell 2k + 1 takes 3/4 u[k] + 1/4 u[k + 1], per axis, where indices -1 and
// n read a halo of linearly extrapolated cells taken on all axes at once:
// halo(a) = 2 u[sym(a)] - u[refl(a)], sym mapping -1 -> 0 and n -> n - 1,
// refl mapping -1 -> 1 and n -> n - 2 on every halo axis of a.
//
// Plain C++ with no CUDA dependency: the device kernels call these
// functions, and a host build of the same header checks their index
// arithmetic against the NumPy statement of the reference.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define MGD_HD __host__ __device__ __forceinline__
#else
#define MGD_HD inline
#endif

namespace odil {
namespace mgd {

struct Grid {
    int dim;        // 1..3 axes
    int cell;       // 0: node refinement, 1: cell refinement
    int64_t n[3];   // coarse sizes, 1 beyond dim
    int64_t m[3];   // fine sizes, 1 beyond dim
};

MGD_HD int64_t fine_size(int64_t n, int cell) { return cell ? 2 * n : 2 * n - 1; }

// Coarse taps of fine coordinate o along one axis: node -> coarse indices,
// cell -> halo indices in [-1, n].
template <typename T>
MGD_HD int fine_taps(int64_t o, int cell, int64_t* a, T* w) {
    const int64_t k = o >> 1;
    if (!cell) {
        a[0] = k;
        if ((o & 1) == 0) {
            w[0] = T(1);
            return 1;
        }
        a[1] = k + 1;
        w[0] = w[1] = T(0.5);
        return 2;
    }
    a[0] = k;
    w[0] = T(0.75);
    a[1] = (o & 1) ? k + 1 : k - 1;
    w[1] = T(0.25);
    return 2;
}

// Value at halo multi-index a of a cell grid.
template <typename T>
MGD_HD T halo_value(const Grid& g, const T* u, const int64_t* a) {
    int64_t is = 0, ir = 0;
    bool halo = false;
    for (int d = 0; d < g.dim; ++d) {
        int64_t s = a[d], r = a[d];
        if (a[d] < 0) {
            s = 0;
            r = 1;
            halo = true;
        } else if (a[d] >= g.n[d]) {
            s = g.n[d] - 1;
            r = g.n[d] - 2;
            halo = true;
        }
        is = is * g.n[d] + s;
        ir = ir * g.n[d] + r;
    }
    if (!halo) return u[is];
    return T(2) * u[is] - u[ir];
}

MGD_HD void unflatten(const int64_t* size, int dim, int64_t i, int64_t* o) {
    for (int d = dim - 1; d >= 0; --d) {
        o[d] = i % size[d];
        i /= size[d];
    }
}

// Refined value at fine multi-index o.
template <typename T>
MGD_HD T refine_point(const Grid& g, const T* u, const int64_t* o) {
    int64_t a[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    T w[3][2] = {{T(1), T(0)}, {T(1), T(0)}, {T(1), T(0)}};
    int nt[3] = {1, 1, 1};
    for (int d = 0; d < g.dim; ++d) nt[d] = fine_taps(o[d], g.cell, a[d], w[d]);
    T acc = T(0);
    for (int c0 = 0; c0 < nt[0]; ++c0)
        for (int c1 = 0; c1 < nt[1]; ++c1)
            for (int c2 = 0; c2 < nt[2]; ++c2) {
                const int64_t aa[3] = {a[0][c0], a[1][c1], a[2][c2]};
                const T ww = w[0][c0] * w[1][c1] * w[2][c2];
                T v;
                if (g.cell) {
                    v = halo_value(g, u, aa);
                } else {
                    int64_t idx = 0;
                    for (int d = 0; d < g.dim; ++d) idx = idx * g.n[d] + aa[d];
                    v = u[idx];
                }
                acc += ww * v;
            }
    return acc;
}

// Fine taps of coarse (node) or halo (cell) coordinate a along one axis,
// clipped to the fine grid [0, m): the fine points whose refinement reads a.
template <typename T>
MGD_HD int coarse_taps(int64_t a, int64_t m, int cell, int64_t* o, T* w) {
    int k = 0;
    if (!cell) {
        const int64_t c[3] = {2 * a - 1, 2 * a, 2 * a + 1};
        const T cw[3] = {T(0.5), T(1), T(0.5)};
        for (int j = 0; j < 3; ++j)
            if (c[j] >= 0 && c[j] < m) {
                o[k] = c[j];
                w[k] = cw[j];
                ++k;
            }
        return k;
    }
    const int64_t c[4] = {2 * a - 1, 2 * a, 2 * a + 1, 2 * a + 2};
    const T cw[4] = {T(0.25), T(0.75), T(0.75), T(0.25)};
    for (int j = 0; j < 4; ++j)
        if (c[j] >= 0 && c[j] < m) {
            o[k] = c[j];
            w[k] = cw[j];
            ++k;
        }
    return k;
}

// sum over fine o of weight(o, a) gf[o], a a coarse or halo multi-index.
template <typename T>
MGD_HD T gather_fine(const Grid& g, const T* gf, const int64_t* a) {
    int64_t o[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    T w[3][4] = {{T(1), T(0), T(0), T(0)}, {T(1), T(0), T(0), T(0)},
                 {T(1), T(0), T(0), T(0)}};
    int nt[3] = {1, 1, 1};
    for (int d = 0; d < g.dim; ++d) nt[d] = coarse_taps(a[d], g.m[d], g.cell, o[d], w[d]);
    T acc = T(0);
    for (int c0 = 0; c0 < nt[0]; ++c0)
        for (int c1 = 0; c1 < nt[1]; ++c1)
            for (int c2 = 0; c2 < nt[2]; ++c2) {
                int64_t idx = 0;
                const int64_t oo[3] = {o[0][c0], o[1][c1], o[2][c2]};
                for (int d = 0; d < g.dim; ++d) idx = idx * g.m[d] + oo[d];
                acc += w[0][c0] * w[1][c1] * w[2][c2] * gf[idx];
            }
    return acc;
}

// Adjoint of the refinement at coarse multi-index q: sum over fine o of
// dP(o)/du(q) gf[o].  For cells, the halo point a contributes through
// 2 [sym(a) = q] - [refl(a) = q]; per axis q is reached from itself, from
// a halo index whose sym is q (q = 0 or n - 1) and from one whose refl is q
// (q = 1 or n - 2), and a combination counts +2 when all its halo axes are
// sym ones, -1 when all are refl ones, 0 when mixed, 1 with no halo axis.
template <typename T>
MGD_HD T refine_adjoint_point(const Grid& g, const T* gf, const int64_t* q) {
    if (!g.cell) return gather_fine(g, gf, q);
    int64_t a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    int kind[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // 0 self, 1 sym, 2 refl
    int nc[3] = {1, 1, 1};
    for (int d = 0; d < g.dim; ++d) {
        const int64_t n = g.n[d], v = q[d];
        int k = 0;
        a[d][k] = v;
        kind[d][k++] = 0;
        if (v == 0) { a[d][k] = -1; kind[d][k++] = 1; }
        if (v == n - 1) { a[d][k] = n; kind[d][k++] = 1; }
        if (v == 1) { a[d][k] = -1; kind[d][k++] = 2; }
        if (v == n - 2) { a[d][k] = n; kind[d][k++] = 2; }
        nc[d] = k;
    }
    T acc = T(0);
    for (int c0 = 0; c0 < nc[0]; ++c0)
        for (int c1 = 0; c1 < nc[1]; ++c1)
            for (int c2 = 0; c2 < nc[2]; ++c2) {
                const int ks[3] = {kind[0][c0], kind[1][c1], kind[2][c2]};
                bool sym = false, refl = false;
                for (int d = 0; d < 3; ++d) {
                    sym = sym || ks[d] == 1;
                    refl = refl || ks[d] == 2;
                }
                if (sym && refl) continue;
                const T coef = sym ? T(2) : (refl ? T(-1) : T(1));
                const int64_t aa[3] = {a[0][c0], a[1][c1], a[2][c2]};
                acc += coef * gather_fine(g, gf, aa);
            }
    return acc;
}

// wf[o] = beta * gf[o] for the fine points o with o >> 1 == q on every axis;
// every fine point is owned by exactly one coarse point.
template <typename T>
MGD_HD void scale_owned(const Grid& g, const T* gf, T* wf, T beta, const int64_t* q) {
    int64_t lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    for (int d = 0; d < g.dim; ++d) {
        lo[d] = 2 * q[d];
        hi[d] = 2 * q[d] + 2 < g.m[d] ? 2 * q[d] + 2 : g.m[d];
    }
    for (int64_t o0 = lo[0]; o0 < hi[0]; ++o0)
        for (int64_t o1 = lo[1]; o1 < hi[1]; ++o1)
            for (int64_t o2 = lo[2]; o2 < hi[2]; ++o2) {
                const int64_t oo[3] = {o0, o1, o2};
                int64_t idx = 0;
                for (int d = 0; d < g.dim; ++d) idx = idx * g.m[d] + oo[d];
                wf[idx] = beta * gf[idx];
            }
}

}  // namespace mgd
}  // namespace odil
