// Steady incompressible Navier-Stokes in the lid-driven cavity: residual and
// Jacobian coefficient fields of the reference operator ns_steady.py:142-433
// with its defaults (--bc 0 no-slip with lid u = 1 at y = 1 by quadratic
// extrapolation, --rhiechow 1, deferred-correction upwind for momentum).
//
// The operator is affine in the live fields (u, v, p) once the frozen copies
// (uf, vf, pf: the state, stop_gradient in the reference) are fixed:
//   F(live) = L(frozen) live + c(frozen).
// Per cell the kernel first collects the frozen context (boundary-extrapolated
// 5-point stencils, their second neighbours, the Rhie-Chow weights g), then
// evaluates the live part.  The residual evaluates it on the state; the
// Jacobian evaluates its linear part (constants dropped) on each of the 15
// unit seeds (field x {c, x-1, x+1, y-1, y+1}), which gives exactly the
// per-shift coefficient fields Problem._eval_grad0 (util_op.py:585-614)
// returns, without cancellation.
#include "common.cuh"

namespace odil {
namespace {

template <typename T>
struct NsDev {
    int n;                 // grid n x n on [0, 1]^2
    T dx, dy, mu;
    T kreg;                // Laplacian penalty weight (0: off)
    T imp_coeff;           // alpha N / n_imp (0: no imposed points)
    const T* mask;         // [n*n] imposed-point mask or null
    const T* u_imp;
    const T* v_imp;
    int pin;               // flat index of the pinned pressure cell, -1: none
    T pin_w;
    int neq;
};

template <typename T>
__device__ __forceinline__ T quadh(T u0, T u1, T u1p) { return (u0 - T(6) * u1 + T(8) * u1p) / T(3); }
template <typename T>
__device__ __forceinline__ T linex(T u0, T u1) { return T(2) * u1 - u0; }

// Stencil [c, x-1, x+1, y-1, y+1] of a raw field at (x, y), periodic roll.
template <typename T>
__device__ __forceinline__ void raw5(const T* a, int n, int x, int y, T* s) {
    const int xm = x == 0 ? n - 1 : x - 1, xp = x + 1 == n ? 0 : x + 1;
    const int ym = y == 0 ? n - 1 : y - 1, yp = y + 1 == n ? 0 : y + 1;
    s[0] = __ldg(a + x * n + y);
    s[1] = __ldg(a + xm * n + y);
    s[2] = __ldg(a + xp * n + y);
    s[3] = __ldg(a + x * n + ym);
    s[4] = __ldg(a + x * n + yp);
}

// Boundary treatments of ns_steady.py:250-273 on a 5-point stencil at (x, y).
// kind 0: u (lid value `top` at y = 1), kind 1: v, kind 2: linear extrap (p).
template <typename T>
__device__ __forceinline__ void bc5(T* s, int n, int x, int y, int kind, T top) {
    if (kind == 2) {
        if (x == 0) s[1] = linex(s[2], s[0]);
        if (x == n - 1) s[2] = linex(s[1], s[0]);
        if (y == 0) s[3] = linex(s[4], s[0]);
        if (y == n - 1) s[4] = linex(s[3], s[0]);
    } else {
        if (x == 0) s[1] = quadh(s[2], s[0], T(0));
        if (x == n - 1) s[2] = quadh(s[1], s[0], T(0));
        if (y == 0) s[3] = quadh(s[4], s[0], T(0));
        if (y == n - 1) s[4] = quadh(s[3], s[0], kind == 0 ? top : T(0));
    }
}

// Boundary-modified stencil of a frozen field at (x, y) plus the second
// neighbours of stencil5 (ns_steady.py:285-296): [xmm, xpp, ymm, ypp].
template <typename T>
__device__ void frozen9(const T* a, int n, int x, int y, int kind, T* s, T* s5) {
    raw5(a, n, x, y, s);
    bc5(s, n, x, y, kind, T(1));
    const int xm = x == 0 ? n - 1 : x - 1, xp = x + 1 == n ? 0 : x + 1;
    const int ym = y == 0 ? n - 1 : y - 1, yp = y + 1 == n ? 0 : y + 1;
    T t[5];
    // roll(st[1], 1, axis 0)[x] = st[1] at cell x-1
    raw5(a, n, xm, y, t);
    bc5(t, n, xm, y, kind, T(1));
    s5[0] = x == 0 ? s[1] : t[1];
    raw5(a, n, xp, y, t);
    bc5(t, n, xp, y, kind, T(1));
    s5[1] = x == n - 1 ? s[2] : t[2];
    raw5(a, n, x, ym, t);
    bc5(t, n, x, ym, kind, T(1));
    s5[2] = y == 0 ? s[3] : t[3];
    raw5(a, n, x, yp, t);
    bc5(t, n, x, yp, kind, T(1));
    s5[3] = y == n - 1 ? s[4] : t[4];
}

template <typename T>
struct Frozen {
    T uf[5], uf5[4], vf[5], vf5[4], pf[5], pf5[4];
    T g, gxm, gxp, gym, gyp;
    // frozen-only terms of fu, fv (deferred correction) and of the fluxes
    T fu_c, fv_c, qxm_c, qxp_c, qym_c, qyp_c;
};

template <typename T>
__device__ __forceinline__ T gval(const NsDev<T>& P, const T* u, const T* v, int x, int y) {
    const int k = x * P.n + y;
    return fabs(__ldg(u + k)) / P.dx + fabs(__ldg(v + k)) / P.dy +
           P.mu * (T(2) / (P.dx * P.dx) + T(2) / (P.dy * P.dy));
}

// upwind_second (ns_steady.py:171-188) x and y derivatives of a frozen field.
template <typename T>
__device__ __forceinline__ void up2(const NsDev<T>& P, int x, int y, const T* s, const T* s5, T uf,
                                    T vf, T* qx, T* qy) {
    const int n = P.n;
    T q_xm = (s5[0] - T(4) * s[1] + T(3) * s[0]) / (T(2) * P.dx);
    T q_xp = (-T(3) * s[0] + T(4) * s[2] - s5[1]) / (T(2) * P.dx);
    T q_ym = (s5[2] - T(4) * s[3] + T(3) * s[0]) / (T(2) * P.dy);
    T q_yp = (-T(3) * s[0] + T(4) * s[4] - s5[3]) / (T(2) * P.dy);
    if (x == 0) q_xm = (s[0] - s[1]) / P.dx;
    if (x == n - 1) q_xp = (s[2] - s[0]) / P.dx;
    if (y == 0) q_ym = (s[0] - s[3]) / P.dy;
    if (y == n - 1) q_yp = (s[4] - s[0]) / P.dy;
    *qx = uf > T(0) ? q_xm : q_xp;
    *qy = vf > T(0) ? q_ym : q_yp;
}

// upwind_low (ns_steady.py:193-202)
template <typename T>
__device__ __forceinline__ void up1(const NsDev<T>& P, const T* s, T uf, T vf, T* qx, T* qy) {
    *qx = uf > T(0) ? (s[0] - s[1]) / P.dx : (s[2] - s[0]) / P.dx;
    *qy = vf > T(0) ? (s[0] - s[3]) / P.dy : (s[4] - s[0]) / P.dy;
}

template <typename T>
__device__ void make_frozen(const NsDev<T>& P, const T* u, const T* v, const T* p, int x, int y,
                            Frozen<T>* F) {
    const int n = P.n;
    frozen9(u, n, x, y, 0, F->uf, F->uf5);
    frozen9(v, n, x, y, 1, F->vf, F->vf5);
    frozen9(p, n, x, y, 2, F->pf, F->pf5);
    const T uf = F->uf[0], vf = F->vf[0];
    T a, b, c1, c2;
    up2(P, x, y, F->uf, F->uf5, uf, vf, &a, &b);
    up1(P, F->uf, uf, vf, &c1, &c2);
    F->fu_c = uf * (a - c1) + vf * (b - c2);
    up2(P, x, y, F->vf, F->vf5, uf, vf, &a, &b);
    up1(P, F->vf, uf, vf, &c1, &c2);
    F->fv_c = uf * (a - c1) + vf * (b - c2);
    const int xm = x == 0 ? n - 1 : x - 1, xp = x + 1 == n ? 0 : x + 1;
    const int ym = y == 0 ? n - 1 : y - 1, yp = y + 1 == n ? 0 : y + 1;
    F->g = gval(P, u, v, x, y);
    F->gxm = gval(P, u, v, xm, y);
    F->gxp = gval(P, u, v, xp, y);
    F->gym = gval(P, u, v, x, ym);
    F->gyp = gval(P, u, v, x, yp);
    const T* pf = F->pf;
    const T* pf5 = F->pf5;
    F->qxm_c = (T(1) / F->gxm * (pf[0] - pf5[0]) / (T(2) * P.dx)) * T(0.5) +
               (T(1) / F->g * (pf[2] - pf[1]) / (T(2) * P.dx)) * T(0.5);
    F->qxp_c = (T(1) / F->gxp * (pf5[1] - pf[0]) / (T(2) * P.dx)) * T(0.5) +
               (T(1) / F->g * (pf[2] - pf[1]) / (T(2) * P.dx)) * T(0.5);
    F->qym_c = (T(1) / F->gym * (pf[0] - pf5[2]) / (T(2) * P.dy)) * T(0.5) +
               (T(1) / F->g * (pf[4] - pf[3]) / (T(2) * P.dy)) * T(0.5);
    F->qyp_c = (T(1) / F->gyp * (pf5[3] - pf[0]) / (T(2) * P.dy)) * T(0.5) +
               (T(1) / F->g * (pf[4] - pf[3]) / (T(2) * P.dy)) * T(0.5);
}

// Live part.  lu, lv, lp: raw live stencils [c, x-1, x+1, y-1, y+1];
// lin = true drops every term that does not multiply a live value (frozen-
// only terms, the lid value, imposed data).  out[neq].
template <typename T>
__device__ void ns_live(const NsDev<T>& P, const Frozen<T>& F, int x, int y, const T* lu_raw,
                        const T* lv_raw, const T* lp_raw, bool lin, T* out) {
    const int n = P.n;
    T lu[5], lv[5], lp[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        lu[k] = lu_raw[k];
        lv[k] = lv_raw[k];
        lp[k] = lp_raw[k];
    }
    bc5(lu, n, x, y, 0, lin ? T(0) : T(1));
    bc5(lv, n, x, y, 1, T(0));
    bc5(lp, n, x, y, 2, T(0));
    const T uf = F.uf[0], vf = F.vf[0];
    T ux, uy, vx, vy;
    up1(P, lu, uf, vf, &ux, &uy);
    up1(P, lv, uf, vf, &vx, &vy);
    const T u_xx = (lu[2] - T(2) * lu[0] + lu[1]) / (P.dx * P.dx);
    const T u_yy = (lu[4] - T(2) * lu[0] + lu[3]) / (P.dy * P.dy);
    const T v_xx = (lv[2] - T(2) * lv[0] + lv[1]) / (P.dx * P.dx);
    const T v_yy = (lv[4] - T(2) * lv[0] + lv[3]) / (P.dy * P.dy);
    const T p_xc = (lp[2] - lp[1]) / (T(2) * P.dx);
    const T p_yc = (lp[4] - lp[3]) / (T(2) * P.dy);
    const T cu = lin ? T(0) : F.fu_c;
    const T cv = lin ? T(0) : F.fv_c;
    out[0] = cu + uf * ux + vf * uy - P.mu * (u_xx + u_yy) + p_xc;
    out[1] = cv + uf * vx + vf * vy - P.mu * (v_xx + v_yy) + p_yc;
    // Rhie-Chow fluxes (ns_steady.py:339-372), zero at the walls (bc = 0).
    const T L = lin ? T(0) : T(1);
    T qxm = (lu[0] + lu[1]) * T(0.5) + L * F.qxm_c -
            (T(1) / F.gxm + T(1) / F.g) * T(0.5) * (lp[0] - lp[1]) / P.dx;
    T qxp = (lu[0] + lu[2]) * T(0.5) + L * F.qxp_c -
            (T(1) / F.gxp + T(1) / F.g) * T(0.5) * (lp[2] - lp[0]) / P.dx;
    T qym = (lv[0] + lv[3]) * T(0.5) + L * F.qym_c -
            (T(1) / F.gym + T(1) / F.g) * T(0.5) * (lp[0] - lp[3]) / P.dy;
    T qyp = (lv[0] + lv[4]) * T(0.5) + L * F.qyp_c -
            (T(1) / F.gyp + T(1) / F.g) * T(0.5) * (lp[4] - lp[0]) / P.dy;
    if (x == 0) qxm = T(0);
    if (x == n - 1) qxp = T(0);
    if (y == 0) qym = T(0);
    if (y == n - 1) qyp = T(0);
    out[2] = (qxp - qxm) / P.dx + (qyp - qym) / P.dy;
    int e = 3;
    if (P.mask) {
        const int k = x * n + y;
        const T m = __ldg(P.mask + k);
        out[e++] = m * (lu_raw[0] - (lin ? T(0) : __ldg(P.u_imp + k))) * P.imp_coeff;
        out[e++] = m * (lv_raw[0] - (lin ? T(0) : __ldg(P.v_imp + k))) * P.imp_coeff;
    }
    if (P.kreg != T(0)) {
        out[e++] = u_xx * P.kreg;
        out[e++] = u_yy * P.kreg;
        out[e++] = v_xx * P.kreg;
        out[e++] = v_yy * P.kreg;
    }
    if (P.pin >= 0) out[e++] = (x * n + y == P.pin ? T(1) : T(0)) * lp_raw[0] * P.pin_w;
}

constexpr int NS_MAXEQ = 10;

template <typename T>
__global__ void __launch_bounds__(128) ns_residual_kernel(NsDev<T> P, const T* __restrict__ u,
                                                          const T* __restrict__ v,
                                                          const T* __restrict__ p,
                                                          T* __restrict__ f) {
    const int n = P.n;
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (y >= n) return;
    Frozen<T> F;
    make_frozen(P, u, v, p, x, y, &F);
    T lu[5], lv[5], lp[5], out[NS_MAXEQ];
    raw5(u, n, x, y, lu);
    raw5(v, n, x, y, lv);
    raw5(p, n, x, y, lp);
    ns_live(P, F, x, y, lu, lv, lp, false, out);
    const int64_t N = (int64_t)n * n;
    for (int e = 0; e < P.neq; ++e) f[e * N + x * n + y] = out[e];
}

// coef[(e * 15 + s) * N + cell]: d f_e / d (live slot s), slot = field*5 + k,
// field in (u, v, p), k in (c, x-1, x+1, y-1, y+1).
template <typename T>
__global__ void __launch_bounds__(128) ns_coef_kernel(NsDev<T> P, const T* __restrict__ u,
                                                      const T* __restrict__ v,
                                                      const T* __restrict__ p,
                                                      T* __restrict__ coef) {
    const int n = P.n;
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = blockIdx.y;
    if (y >= n) return;
    Frozen<T> F;
    make_frozen(P, u, v, p, x, y, &F);
    const int64_t N = (int64_t)n * n;
    const int64_t cell = (int64_t)x * n + y;
    for (int s = 0; s < 15; ++s) {
        T lu[5] = {0, 0, 0, 0, 0}, lv[5] = {0, 0, 0, 0, 0}, lp[5] = {0, 0, 0, 0, 0};
        const int fld = s / 5, k = s % 5;
        if (fld == 0) lu[k] = T(1);
        else if (fld == 1) lv[k] = T(1);
        else lp[k] = T(1);
        T out[NS_MAXEQ];
        ns_live(P, F, x, y, lu, lv, lp, true, out);
        for (int e = 0; e < P.neq; ++e) coef[((int64_t)e * 15 + s) * N + cell] = out[e];
    }
}

template <typename T>
int make_ns(const odil_ns_params* q, NsDev<T>* P) {
    if (!q) return ODIL_ERR_ARG;
    if (q->n < 3 || q->n > 65535) return ODIL_ERR_SHAPE;
    if (!(q->re > 0)) return ODIL_ERR_ARG;
    P->n = (int)q->n;
    P->dx = P->dy = (T)(1.0 / q->n);
    P->mu = (T)(1.0 / q->re);
    P->kreg = (T)q->kreg;
    P->mask = (const T*)q->mask;
    P->u_imp = (const T*)q->u_imp;
    P->v_imp = (const T*)q->v_imp;
    P->imp_coeff = (T)q->imp_coeff;
    if (q->mask && (!q->u_imp || !q->v_imp)) return ODIL_ERR_ARG;
    P->pin = q->pin >= 0 ? (int)q->pin : -1;
    if (q->pin >= q->n * q->n) return ODIL_ERR_SHAPE;
    P->pin_w = (T)q->pin_weight;
    P->neq = 3 + (q->mask ? 2 : 0) + (q->kreg != 0 ? 4 : 0) + (q->pin >= 0 ? 1 : 0);
    return ODIL_OK;
}

template <typename T>
int residual_impl(const odil_ns_params* q, const T* u, const T* v, const T* p, T* f,
                  void* stream) {
    NsDev<T> P;
    int st = make_ns<T>(q, &P);
    if (st) return st;
    if (!u || !v || !p || !f) return ODIL_ERR_ARG;
    dim3 block(128), grid((P.n + 127) / 128, P.n);
    ns_residual_kernel<T><<<grid, block, 0, as_stream(stream)>>>(P, u, v, p, f);
    return launch_status();
}

template <typename T>
int coef_impl(const odil_ns_params* q, const T* u, const T* v, const T* p, T* coef,
              void* stream) {
    NsDev<T> P;
    int st = make_ns<T>(q, &P);
    if (st) return st;
    if (!u || !v || !p || !coef) return ODIL_ERR_ARG;
    dim3 block(128), grid((P.n + 127) / 128, P.n);
    ns_coef_kernel<T><<<grid, block, 0, as_stream(stream)>>>(P, u, v, p, coef);
    return launch_status();
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_ns_num_equations(const odil_ns_params* q) {
    NsDev<double> P;
    int st = make_ns<double>(q, &P);
    return st ? st : P.neq;
}
ODIL_API int odil_ns_residual_f32(const odil_ns_params* q, const float* u, const float* v,
                                  const float* p, float* f, void* stream) {
    return residual_impl<float>(q, u, v, p, f, stream);
}
ODIL_API int odil_ns_residual_f64(const odil_ns_params* q, const double* u, const double* v,
                                  const double* p, double* f, void* stream) {
    return residual_impl<double>(q, u, v, p, f, stream);
}
ODIL_API int odil_ns_jacobian_f32(const odil_ns_params* q, const float* u, const float* v,
                                  const float* p, float* coef, void* stream) {
    return coef_impl<float>(q, u, v, p, coef, stream);
}
ODIL_API int odil_ns_jacobian_f64(const odil_ns_params* q, const double* u, const double* v,
                                  const double* p, double* coef, void* stream) {
    return coef_impl<double>(q, u, v, p, coef, stream);
}
