// Operators in stencil form on the GPU: the data model of the reference's
// SparseOperator (multigrid.py:877-1214) -- a list of shifts s with one
// coefficient field C_s on the output grid --
//     (A u)[c] = sum_s C_s[c] u[stride c + s]     (zero outside the grid, or
//                                                   wrapped on periodic axes)
// with the products the multigrid needs: A u (mul_field 958-969), A^T u
// (mul_transpose_field 1006-1027, stride 1 and 2), A^T B as a stencil
// (mul_transpose_op 1035-1071), the Galerkin coarse operator R A T
// (multigrid.py:125-131; coarsen_sparse_operator 390-427 in stencil form),
// and damped Jacobi sweeps over block systems (smoother_jacobi 543-552).
// Grids have up to three axes; axes beyond `dim` have size 1.
#include "common.cuh"

namespace odil {
namespace {

constexpr int MAXS = ODIL_STENCIL_MAXS;

struct StDev {
    int dim, stride, ns;
    int per[3];
    int nw[3], nwh[3];
    signed char sh[MAXS][3];
    int64_t nh;  // output cells
};

int make_st(const odil_stencil* A, StDev* d) {
    if (!A) return ODIL_ERR_ARG;
    if (A->dim < 1 || A->dim > 3 || (A->stride != 1 && A->stride != 2) || A->nshift < 0 ||
        A->nshift > MAXS)
        return ODIL_ERR_SHAPE;
    d->dim = A->dim;
    d->stride = A->stride;
    d->ns = A->nshift;
    int64_t nh = 1;
    for (int a = 0; a < 3; ++a) {
        const int64_t n = a < A->dim ? A->nw[a] : 1;
        if (n < 1 || n > (1 << 30)) return ODIL_ERR_SHAPE;
        d->nw[a] = (int)n;
        d->per[a] = a < A->dim ? (A->periodic[a] ? 1 : 0) : 0;
        int nhh;
        if (a >= A->dim) {
            nhh = 1;
        } else if (d->per[a] && A->stride == 2) {
            if (n % 2) return ODIL_ERR_SHAPE;
            nhh = (int)(n / 2);
        } else {
            nhh = (int)((n - 1) / A->stride + 1);
        }
        d->nwh[a] = nhh;
        nh *= nhh;
    }
    if (nh > (int64_t(1) << 31) - 1) return ODIL_ERR_SHAPE;
    d->nh = nh;
    for (int s = 0; s < A->nshift; ++s) {
        for (int a = 0; a < 3; ++a) {
            const int v = a < A->dim ? A->shifts[s][a] : 0;
            if (v < -8 || v > 8) return ODIL_ERR_SHAPE;
            d->sh[s][a] = (signed char)v;
        }
    }
    return ODIL_OK;
}

__device__ __forceinline__ void unflat(int64_t k, const int* n, int* c) {
    c[2] = (int)(k % n[2]);
    k /= n[2];
    c[1] = (int)(k % n[1]);
    c[0] = (int)(k / n[1]);
}

__device__ __forceinline__ int64_t flat(const int* c, const int* n) {
    return ((int64_t)c[0] * n[1] + c[1]) * n[2] + c[2];
}

// Index e = stride * c + s along every axis; false if outside a
// non-periodic axis.
__device__ __forceinline__ bool src_index(const StDev& A, const int* c, int s, int* e) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int v = A.stride * c[a] + A.sh[s][a];
        const int n = A.nw[a];
        if (A.per[a]) {
            v = v < 0 ? v + n : (v >= n ? v - n : v);
            if (v < 0 || v >= n) v = ((v % n) + n) % n;
        } else if (v < 0 || v >= n) {
            return false;
        }
        e[a] = v;
    }
    return true;
}

// out[c] = beta * out[c] + alpha * sum_s C_s[c] u[stride c + s]
template <typename T>
__global__ void __launch_bounds__(256) st_apply_kernel(StDev A, const T* __restrict__ coef,
                                                       const T* __restrict__ u, T* __restrict__ out,
                                                       T alpha, T beta) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.nh) return;
    int c[3];
    unflat(k, A.nwh, c);
    T s = T(0);
    for (int q = 0; q < A.ns; ++q) {
        int e[3];
        if (src_index(A, c, q, e)) s += __ldg(coef + q * A.nh + k) * __ldg(u + flat(e, A.nw));
    }
    out[k] = (beta == T(0) ? T(0) : beta * out[k]) + alpha * s;
}

// out[e] = beta * out[e] + alpha * sum_{s, c : stride c + s = e} C_s[c] uh[c]
// (gather over the fine grid: for each shift, c = (e - s) / stride when
// divisible and inside the coarse grid, wrapped on periodic axes).
template <typename T>
__global__ void __launch_bounds__(256) st_apply_t_kernel(StDev A, const T* __restrict__ coef,
                                                         const T* __restrict__ uh,
                                                         T* __restrict__ out, T alpha, T beta) {
    int64_t nf = (int64_t)A.nw[0] * A.nw[1] * A.nw[2];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nf) return;
    int e[3];
    unflat(k, A.nw, e);
    T s = T(0);
    for (int q = 0; q < A.ns; ++q) {
        int c[3];
        bool ok = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int d = e[a] - A.sh[q][a];
            const int n = A.nw[a];
            if (A.per[a]) d = ((d % n) + n) % n;
            if (d < 0 || d % A.stride) { ok = false; break; }
            const int cc = d / A.stride;
            if (cc >= A.nwh[a]) { ok = false; break; }
            // The entry exists only if stride*cc + s lands back on e (not on a
            // wrapped copy outside a non-periodic range).
            c[a] = cc;
        }
        if (ok) {
            const int64_t kc = flat(c, A.nwh);
            s += __ldg(coef + q * A.nh + kc) * __ldg(uh + kc);
        }
    }
    out[k] = (beta == T(0) ? T(0) : beta * out[k]) + alpha * s;
}

// A^T B as a stride-1 stencil, coefficient fields of the reference's
// mul_transpose_op: for every pair (a, b) with b - a = d,
//   res_d[e] += (C^A_a * C^B_b)[e - a]      (zero outside / wrapped).
// pair_d[q] = index of shift d of the pair list; one thread per (cell, d).
struct PairList {
    int npair;
    short ia[MAXS * 32], ib[MAXS * 32], id[MAXS * 32];
};

template <typename T>
__global__ void __launch_bounds__(256) st_mul_transpose_op_kernel(
    StDev A, const T* __restrict__ ca, StDev B, const T* __restrict__ cb,
    const PairList* __restrict__ pairs, int nd, T* __restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.nh) return;
    int e[3];
    unflat(k, A.nw, e);
    for (int q = 0; q < nd; ++q) out[q * A.nh + k] = T(0);
    for (int p = 0; p < pairs->npair; ++p) {
        const int a = pairs->ia[p], b = pairs->ib[p], d = pairs->id[p];
        int src[3];
        bool ok = true;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            int v = e[ax] - A.sh[a][ax];
            const int n = A.nw[ax];
            if (A.per[ax]) {
                v = ((v % n) + n) % n;
            } else if (v < 0 || v >= n) {
                ok = false;
                break;
            }
            src[ax] = v;
        }
        if (ok) {
            const int64_t ks = flat(src, A.nw);
            out[d * A.nh + k] += __ldg(ca + a * A.nh + ks) * __ldg(cb + b * B.nh + ks);
        }
    }
}

// Galerkin coarse operator Ac_d[C] = sum_{r, a} R_r[C] A_a[2C + r] TT_t[C + d],
// t = r + a - 2d, every index checked against its grid (or wrapped).  dmap
// maps a coarse shift d (offset by DOFF per axis) to its output slot.
constexpr int DOFF = 4;
constexpr int DSPAN = 2 * DOFF + 1;

struct DMap {
    short slot[DSPAN * DSPAN * DSPAN];
    short tslot[3 * 3 * 3];  // TT shift (t + 1 per axis) -> TT field index or -1
};

template <typename T>
__global__ void __launch_bounds__(128) st_galerkin_kernel(StDev R, const T* __restrict__ cr,
                                                          StDev A, const T* __restrict__ ca,
                                                          StDev TT, const T* __restrict__ ct,
                                                          const DMap* __restrict__ dm, int nd,
                                                          T* __restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R.nh) return;
    int C[3];
    unflat(k, R.nwh, C);
    for (int q = 0; q < nd; ++q) out[q * R.nh + k] = T(0);
    for (int r = 0; r < R.ns; ++r) {
        int e[3];
        if (!src_index(R, C, r, e)) continue;
        const T rv = __ldg(cr + r * R.nh + k);
        if (rv == T(0)) continue;
        const int64_t ke = flat(e, A.nw);
        for (int a = 0; a < A.ns; ++a) {
            // e2 = e + a must be inside the fine grid (or wrapped).
            bool ok = true;
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const int v = e[ax] + A.sh[a][ax];
                if (!A.per[ax] && (v < 0 || v >= A.nw[ax])) ok = false;
            }
            if (!ok) continue;
            const T av = __ldg(ca + a * A.nh + ke);
            if (av == T(0)) continue;
            // q_ax = r + a; d_ax with t = q - 2 d in [-1, 1]: 1 or 2 choices.
            int qv[3], dlo[3], dhi[3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                qv[ax] = R.sh[r][ax] + A.sh[a][ax];
                // d in [ceil((q-1)/2), floor((q+1)/2)]
                const int lo2 = qv[ax] - 1, hi2 = qv[ax] + 1;
                dlo[ax] = lo2 >= 0 ? (lo2 + 1) / 2 : -((-lo2) / 2);
                dhi[ax] = hi2 >= 0 ? hi2 / 2 : -((-hi2 + 1) / 2);
            }
            for (int d0 = dlo[0]; d0 <= dhi[0]; ++d0)
                for (int d1 = dlo[1]; d1 <= dhi[1]; ++d1)
                    for (int d2 = dlo[2]; d2 <= dhi[2]; ++d2) {
                        const int dd[3] = {d0, d1, d2};
                        int t[3], C2[3];
                        bool ok2 = true;
#pragma unroll
                        for (int ax = 0; ax < 3; ++ax) {
                            t[ax] = qv[ax] - 2 * dd[ax];
                            int v = C[ax] + dd[ax];
                            const int n = R.nwh[ax];
                            if (TT.per[ax]) {
                                v = ((v % n) + n) % n;
                            } else if (v < 0 || v >= n) {
                                ok2 = false;
                            }
                            C2[ax] = v;
                            if (dd[ax] < -DOFF || dd[ax] > DOFF) ok2 = false;
                        }
                        if (!ok2) continue;
                        const int ts = dm->tslot[((t[0] + 1) * 3 + (t[1] + 1)) * 3 + (t[2] + 1)];
                        if (ts < 0) continue;
                        const int slot =
                            dm->slot[((d0 + DOFF) * DSPAN + (d1 + DOFF)) * DSPAN + (d2 + DOFF)];
                        if (slot < 0) continue;
                        const T tv = __ldg(ct + ts * TT.nh + flat(C2, TT.nwh));
                        out[slot * R.nh + k] += rv * av * tv;
                    }
        }
    }
}

// Block damped Jacobi / residual for nvar coupled fields on one grid:
//   r_i = f_i - sum_j A_ij u_j;   u_out_i = u_i + omega r_i / diag(A_ii)
// One launch per output field i; the terms of row i are passed by value.
constexpr int MAXV = 4;
struct RowTerms {
    int nterm;
    StDev op[MAXV];
    const void* coef[MAXV];
    const void* u[MAXV];
};

template <typename T>
__global__ void __launch_bounds__(256) st_block_row_kernel(RowTerms row, const T* __restrict__ f,
                                                           const T* __restrict__ ui,
                                                           const T* __restrict__ diag,
                                                           T* __restrict__ uout,
                                                           T* __restrict__ rout, T omega) {
    const StDev& A0 = row.op[0];
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A0.nh) return;
    int c[3];
    unflat(k, A0.nwh, c);
    T s = f ? __ldg(f + k) : T(0);
    for (int t = 0; t < row.nterm; ++t) {
        const StDev& A = row.op[t];
        const T* cf = (const T*)row.coef[t];
        const T* u = (const T*)row.u[t];
        for (int q = 0; q < A.ns; ++q) {
            int e[3];
            if (src_index(A, c, q, e)) s -= __ldg(cf + q * A.nh + k) * __ldg(u + flat(e, A.nw));
        }
    }
    if (rout) rout[k] = s;
    if (uout) uout[k] = __ldg(ui + k) + omega * s / __ldg(diag + k);
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

template <typename T>
int apply_impl(const odil_stencil* A, const T* u, T* out, double alpha, double beta,
               void* stream) {
    StDev d;
    int st = make_st(A, &d);
    if (st) return st;
    if (!u || !out || (!A->coef && d.ns)) return ODIL_ERR_ARG;
    st_apply_kernel<T><<<blocks_for(d.nh, 256), 256, 0, as_stream(stream)>>>(
        d, (const T*)A->coef, u, out, (T)alpha, (T)beta);
    return launch_status();
}

template <typename T>
int apply_t_impl(const odil_stencil* A, const T* uh, T* out, double alpha, double beta,
                 void* stream) {
    StDev d;
    int st = make_st(A, &d);
    if (st) return st;
    if (!uh || !out || (!A->coef && d.ns)) return ODIL_ERR_ARG;
    const int64_t nf = (int64_t)d.nw[0] * d.nw[1] * d.nw[2];
    st_apply_t_kernel<T><<<blocks_for(nf, 256), 256, 0, as_stream(stream)>>>(
        d, (const T*)A->coef, uh, out, (T)alpha, (T)beta);
    return launch_status();
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_stencil_apply_f32(const odil_stencil* A, const float* u, float* out,
                                    double alpha, double beta, void* stream) {
    return apply_impl<float>(A, u, out, alpha, beta, stream);
}
ODIL_API int odil_stencil_apply_f64(const odil_stencil* A, const double* u, double* out,
                                    double alpha, double beta, void* stream) {
    return apply_impl<double>(A, u, out, alpha, beta, stream);
}
ODIL_API int odil_stencil_apply_t_f32(const odil_stencil* A, const float* uh, float* out,
                                      double alpha, double beta, void* stream) {
    return apply_t_impl<float>(A, uh, out, alpha, beta, stream);
}
ODIL_API int odil_stencil_apply_t_f64(const odil_stencil* A, const double* uh, double* out,
                                      double alpha, double beta, void* stream) {
    return apply_t_impl<double>(A, uh, out, alpha, beta, stream);
}

// Pairs (a, b) of shifts and the output shift list are computed on the host
// (the caller passes the output stencil `C` with its shifts = all distinct
// b - a); the pair list travels in a small device buffer the caller provides
// (workspace of odil_stencil_pair_workspace_bytes()).
ODIL_API int64_t odil_stencil_pair_workspace_bytes(void) {
    return (int64_t)sizeof(PairList) > (int64_t)sizeof(DMap) ? (int64_t)sizeof(PairList)
                                                              : (int64_t)sizeof(DMap);
}

template <typename T>
static int mto_impl(const odil_stencil* A, const odil_stencil* B, odil_stencil* C, void* ws,
                    int64_t ws_bytes, void* stream) {
    StDev a, b, c;
    int st = make_st(A, &a);
    if (!st) st = make_st(B, &b);
    if (!st) st = make_st(C, &c);
    if (st) return st;
    if (a.stride != 1 || b.stride != 1 || c.stride != 1) return ODIL_ERR_SHAPE;
    for (int ax = 0; ax < 3; ++ax)
        if (a.nw[ax] != b.nw[ax] || a.nw[ax] != c.nw[ax]) return ODIL_ERR_SHAPE;
    if (!ws || ws_bytes < (int64_t)sizeof(PairList)) return ODIL_ERR_WORKSPACE;
    if (!A->coef || !B->coef || !C->coef) return ODIL_ERR_ARG;
    static PairList pl;  // ~24 KB: keep it off the stack (set-up path, one host thread)
    pl.npair = 0;
    for (int i = 0; i < a.ns; ++i)
        for (int j = 0; j < b.ns; ++j) {
            int d = -1;
            for (int q = 0; q < c.ns; ++q) {
                bool eq = true;
                for (int ax = 0; ax < 3; ++ax)
                    if (c.sh[q][ax] != b.sh[j][ax] - a.sh[i][ax]) eq = false;
                if (eq) { d = q; break; }
            }
            if (d < 0) return ODIL_ERR_SHAPE;  // C must list every b - a
            if (pl.npair >= MAXS * 32) return ODIL_ERR_SHAPE;
            pl.ia[pl.npair] = (short)i;
            pl.ib[pl.npair] = (short)j;
            pl.id[pl.npair] = (short)d;
            ++pl.npair;
        }
    cudaStream_t s = as_stream(stream);
    cudaMemcpyAsync(ws, &pl, sizeof(PairList), cudaMemcpyHostToDevice, s);
    st_mul_transpose_op_kernel<T><<<blocks_for(a.nh, 256), 256, 0, s>>>(
        a, (const T*)A->coef, b, (const T*)B->coef, (const PairList*)ws, c.ns, (T*)C->coef);
    // The pair list lives in pageable host memory: wait for the copy before
    // returning (the call is setup, once per operator).
    cudaStreamSynchronize(s);
    return launch_status();
}

ODIL_API int odil_stencil_mul_transpose_op_f32(const odil_stencil* A, const odil_stencil* B,
                                               odil_stencil* C, void* workspace,
                                               int64_t workspace_bytes, void* stream) {
    return mto_impl<float>(A, B, C, workspace, workspace_bytes, stream);
}
ODIL_API int odil_stencil_mul_transpose_op_f64(const odil_stencil* A, const odil_stencil* B,
                                               odil_stencil* C, void* workspace,
                                               int64_t workspace_bytes, void* stream) {
    return mto_impl<double>(A, B, C, workspace, workspace_bytes, stream);
}

template <typename T>
static int galerkin_impl(const odil_stencil* R, const odil_stencil* A, const odil_stencil* TT,
                         odil_stencil* Ac, void* ws, int64_t ws_bytes, void* stream) {
    StDev r, a, t, c;
    int st = make_st(R, &r);
    if (!st) st = make_st(A, &a);
    if (!st) st = make_st(TT, &t);
    if (!st) st = make_st(Ac, &c);
    if (st) return st;
    if (r.stride != 2 || t.stride != 2 || a.stride != 1 || c.stride != 1) return ODIL_ERR_SHAPE;
    for (int ax = 0; ax < 3; ++ax) {
        if (r.nw[ax] != a.nw[ax] || t.nw[ax] != a.nw[ax] || c.nw[ax] != r.nwh[ax] ||
            r.per[ax] != a.per[ax] || t.per[ax] != a.per[ax])
            return ODIL_ERR_SHAPE;
    }
    if (!ws || ws_bytes < (int64_t)sizeof(DMap)) return ODIL_ERR_WORKSPACE;
    if (!R->coef || !A->coef || !TT->coef || !Ac->coef) return ODIL_ERR_ARG;
    DMap dm;
    for (int q = 0; q < DSPAN * DSPAN * DSPAN; ++q) dm.slot[q] = -1;
    for (int q = 0; q < 27; ++q) dm.tslot[q] = -1;
    for (int q = 0; q < c.ns; ++q) {
        int idx = 0;
        for (int ax = 0; ax < 3; ++ax) {
            const int v = c.sh[q][ax];
            if (v < -DOFF || v > DOFF) return ODIL_ERR_SHAPE;
            idx = idx * DSPAN + (v + DOFF);
        }
        dm.slot[idx] = (short)q;
    }
    for (int q = 0; q < t.ns; ++q) {
        int idx = 0;
        for (int ax = 0; ax < 3; ++ax) {
            const int v = t.sh[q][ax];
            if (v < -1 || v > 1) return ODIL_ERR_SHAPE;
            idx = idx * 3 + (v + 1);
        }
        dm.tslot[idx] = (short)q;
    }
    cudaStream_t s = as_stream(stream);
    cudaMemcpyAsync(ws, &dm, sizeof(DMap), cudaMemcpyHostToDevice, s);
    st_galerkin_kernel<T><<<blocks_for(r.nh, 128), 128, 0, s>>>(
        r, (const T*)R->coef, a, (const T*)A->coef, t, (const T*)TT->coef, (const DMap*)ws, c.ns,
        (T*)Ac->coef);
    cudaStreamSynchronize(s);
    return launch_status();
}

ODIL_API int odil_stencil_galerkin_f32(const odil_stencil* R, const odil_stencil* A,
                                       const odil_stencil* TT, odil_stencil* Ac, void* workspace,
                                       int64_t workspace_bytes, void* stream) {
    return galerkin_impl<float>(R, A, TT, Ac, workspace, workspace_bytes, stream);
}
ODIL_API int odil_stencil_galerkin_f64(const odil_stencil* R, const odil_stencil* A,
                                       const odil_stencil* TT, odil_stencil* Ac, void* workspace,
                                       int64_t workspace_bytes, void* stream) {
    return galerkin_impl<double>(R, A, TT, Ac, workspace, workspace_bytes, stream);
}

template <typename T>
static int block_row_impl(int nterm, const odil_stencil* const* ops, const void* const* us,
                          const T* f, const T* ui, const T* diag, T* uout, T* rout, double omega,
                          void* stream) {
    if (nterm < 1 || nterm > MAXV) return ODIL_ERR_SHAPE;
    if (!ops || !us || (!uout && !rout) || (uout && (!ui || !diag))) return ODIL_ERR_ARG;
    RowTerms row;
    row.nterm = nterm;
    for (int t = 0; t < nterm; ++t) {
        int st = make_st(ops[t], &row.op[t]);
        if (st) return st;
        if (row.op[t].stride != 1) return ODIL_ERR_SHAPE;
        for (int ax = 0; ax < 3; ++ax)
            if (row.op[t].nw[ax] != row.op[0].nw[ax]) return ODIL_ERR_SHAPE;
        if (!us[t] || (!ops[t]->coef && row.op[t].ns)) return ODIL_ERR_ARG;
        row.coef[t] = ops[t]->coef;
        row.u[t] = us[t];
    }
    st_block_row_kernel<T><<<blocks_for(row.op[0].nh, 256), 256, 0, as_stream(stream)>>>(
        row, f, ui, diag, uout, rout, (T)omega);
    return launch_status();
}

ODIL_API int odil_stencil_block_row_f32(int nterm, const odil_stencil* const* ops,
                                        const void* const* us, const float* f, const float* u_i,
                                        const float* diag, float* u_out, float* r_out,
                                        double omega, void* stream) {
    return block_row_impl<float>(nterm, ops, us, f, u_i, diag, u_out, r_out, omega, stream);
}
ODIL_API int odil_stencil_block_row_f64(int nterm, const odil_stencil* const* ops,
                                        const void* const* us, const double* f,
                                        const double* u_i, const double* diag, double* u_out,
                                        double* r_out, double omega, void* stream) {
    return block_row_impl<double>(nterm, ops, us, f, u_i, diag, u_out, r_out, omega, stream);
}
