// Device-side scalars and fused vector updates of BiCGStab (van der Vorst,
// right-preconditioned as in the advection Newton solve): the step scalars
// are formed from the dot products on the device, so the solver reads back
// only the two residual norms it tests per iteration, and each update reads
// and writes every vector once.
//
// Scalar array sc (FP64): [0] rho, [1] alpha, [2] omega, [3] beta.
#include "common.cuh"

namespace odil {
namespace {

constexpr int KT = 256;

// phase 0: rho' = dots[0] (= <r^, r>), beta = (rho'/rho)(alpha/omega), rho = rho'
// phase 1: alpha = rho / dots[0] (= <r^, v>)
// phase 2: omega = dots[1] / dots[0] (= <t, s> / <t, t>; dots from one
//          multi-dot of t against (t, s)); omega = 0 when <t, t> is zero or
//          the quotient is not finite, so the update keeps the valid half
//          step x += alpha ph, r = s, and the breakdown shows up as a
//          non-finite norm of s in the next iteration, before x changes.
__global__ void bicg_scalars_kernel(const double* __restrict__ dots, double* __restrict__ sc,
                                    int phase) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (phase == 0) {
        const double rho1 = dots[0];
        sc[3] = (rho1 / sc[0]) * (sc[1] / sc[2]);
        sc[0] = rho1;
    } else if (phase == 1) {
        sc[1] = sc[0] / dots[0];
    } else {
        const double w = dots[1] / dots[0];
        sc[2] = (dots[0] > 0.0 && isfinite(w)) ? w : 0.0;
    }
}

__device__ __forceinline__ float4 ld4(const float* p, int64_t i) {
    return __ldg(reinterpret_cast<const float4*>(p) + i);
}
__device__ __forceinline__ void st4(float* p, int64_t i, float4 v) {
    reinterpret_cast<float4*>(p)[i] = v;
}

// p = r + beta (p - omega v)
__global__ void __launch_bounds__(KT) bicg_p_kernel(float* __restrict__ p,
                                                    const float* __restrict__ r,
                                                    const float* __restrict__ v,
                                                    const double* __restrict__ sc, int64_t n4) {
    const float beta = (float)sc[3], w = (float)sc[2];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 pr = ld4(p, i), rr = ld4(r, i), vv = ld4(v, i);
        float4 o;
        o.x = rr.x + beta * (pr.x - w * vv.x);
        o.y = rr.y + beta * (pr.y - w * vv.y);
        o.z = rr.z + beta * (pr.z - w * vv.z);
        o.w = rr.w + beta * (pr.w - w * vv.w);
        st4(p, i, o);
    }
}

// s = r - alpha v
__global__ void __launch_bounds__(KT) bicg_s_kernel(float* __restrict__ s,
                                                    const float* __restrict__ r,
                                                    const float* __restrict__ v,
                                                    const double* __restrict__ sc, int64_t n4) {
    const float alpha = (float)sc[1];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 rr = ld4(r, i), vv = ld4(v, i);
        float4 o;
        o.x = rr.x - alpha * vv.x;
        o.y = rr.y - alpha * vv.y;
        o.z = rr.z - alpha * vv.z;
        o.w = rr.w - alpha * vv.w;
        st4(s, i, o);
    }
}

// x += alpha ph (+ omega sh);  r = s - omega t   (with_s: the full step)
__global__ void __launch_bounds__(KT) bicg_xr_kernel(float* __restrict__ x, float* __restrict__ r,
                                                     const float* __restrict__ ph,
                                                     const float* __restrict__ sh,
                                                     const float* __restrict__ s,
                                                     const float* __restrict__ t,
                                                     const double* __restrict__ sc, int64_t n4,
                                                     bool with_s) {
    const float alpha = (float)sc[1], w = (float)sc[2];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        float4 xx = ld4(x, i);
        const float4 pp = ld4(ph, i);
        xx.x += alpha * pp.x;
        xx.y += alpha * pp.y;
        xx.z += alpha * pp.z;
        xx.w += alpha * pp.w;
        if (with_s) {
            const float4 ss = ld4(sh, i), s4 = ld4(s, i), tt = ld4(t, i);
            xx.x += w * ss.x;
            xx.y += w * ss.y;
            xx.z += w * ss.z;
            xx.w += w * ss.w;
            float4 rr;
            rr.x = s4.x - w * tt.x;
            rr.y = s4.y - w * tt.y;
            rr.z = s4.z - w * tt.z;
            rr.w = s4.w - w * tt.w;
            st4(r, i, rr);
        }
        st4(x, i, xx);
    }
}

inline unsigned kblocks(int64_t n4) {
    int64_t b = (n4 + KT - 1) / KT;
    const int64_t cap = 152 * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

bool ok16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_bicgstab_scalars(const double* dots, double* sc, int32_t phase, void* stream) {
    if (!dots || !sc || phase < 0 || phase > 2) return ODIL_ERR_ARG;
    bicg_scalars_kernel<<<1, 32, 0, as_stream(stream)>>>(dots, sc, phase);
    return launch_status();
}

ODIL_API int odil_bicgstab_update_p(float* p, const float* r, const float* v, const double* sc,
                                    int64_t n, void* stream) {
    if (n < 1 || n % 4) return ODIL_ERR_SHAPE;
    if (!p || !r || !v || !sc) return ODIL_ERR_ARG;
    if (!ok16(p) || !ok16(r) || !ok16(v)) return ODIL_ERR_ALIGN;
    bicg_p_kernel<<<kblocks(n / 4), KT, 0, as_stream(stream)>>>(p, r, v, sc, n / 4);
    return launch_status();
}

ODIL_API int odil_bicgstab_update_s(float* s, const float* r, const float* v, const double* sc,
                                    int64_t n, void* stream) {
    if (n < 1 || n % 4) return ODIL_ERR_SHAPE;
    if (!s || !r || !v || !sc) return ODIL_ERR_ARG;
    if (!ok16(s) || !ok16(r) || !ok16(v)) return ODIL_ERR_ALIGN;
    bicg_s_kernel<<<kblocks(n / 4), KT, 0, as_stream(stream)>>>(s, r, v, sc, n / 4);
    return launch_status();
}

ODIL_API int odil_bicgstab_update_xr(float* x, float* r, const float* ph, const float* sh,
                                     const float* s, const float* t, const double* sc, int64_t n,
                                     int32_t with_s, void* stream) {
    if (n < 1 || n % 4) return ODIL_ERR_SHAPE;
    if (!x || !ph || !sc || (with_s && (!r || !sh || !s || !t))) return ODIL_ERR_ARG;
    if (!ok16(x) || !ok16(ph) || (with_s && (!ok16(r) || !ok16(sh) || !ok16(s) || !ok16(t))))
        return ODIL_ERR_ALIGN;
    bicg_xr_kernel<<<kblocks(n / 4), KT, 0, as_stream(stream)>>>(x, r, ph, sh, s, t, sc, n / 4,
                                                                 with_s != 0);
    return launch_status();
}
