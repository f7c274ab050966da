// Vector kernels of the optimizers: fused Adam update, deterministic dot and
// multi-dot products, linear combinations (L-BFGS compact direction), axpby.
//
// Reference: optimizer.py:301-314 (AdamNativeOptimizer update, the Keras Adam
// equations), optimizer.py:61-99 (L-BFGS-B with m = 50 correction pairs, run
// here in the compact representation of Byrd, Nocedal & Schnabel 1994).
// All passes are HBM-bound streaming loops with 16-byte vector accesses where
// the pointers allow it.
#include "common.cuh"

namespace odil {
namespace {

constexpr int VT = 256;  // threads per block of the streaming kernels

inline int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 132;
    }
    return n;
}

inline int stream_blocks(int64_t n, int per_thread) {
    int64_t need = (n + (int64_t)VT * per_thread - 1) / ((int64_t)VT * per_thread);
    int64_t cap = (int64_t)sm_count() * 8;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

template <typename T>
struct Vec;
template <>
struct Vec<float> {
    using V = float4;
    static constexpr int W = 4;
};
template <>
struct Vec<double> {
    using V = double2;
    static constexpr int W = 2;
};

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// ---------------------------------------------------------------------------
// Adam (optimizer.py:301-314):
//   m += (g - m)(1 - b1);  v += (g^2 - v)(1 - b2);  x -= alpha m / (sqrt(v) + eps)
template <typename T>
__device__ __forceinline__ void adam1(T& x, T g, T& m, T& v, T alpha, T b1c, T b2c, T eps) {
    m += (g - m) * b1c;
    v += (g * g - v) * b2c;
    x -= (m * alpha) / (sqrt(v) + eps);
}

template <typename T>
__global__ void __launch_bounds__(VT) adam_kernel(T* __restrict__ x, const T* __restrict__ g,
                                                  T* __restrict__ m, T* __restrict__ v,
                                                  int64_t n, T alpha, T b1c, T b2c, T eps,
                                                  bool vec) {
    using V = typename Vec<T>::V;
    constexpr int W = Vec<T>::W;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nv = vec ? n / W : 0;
    for (int64_t i = tid; i < nv; i += stride) {
        V xv = reinterpret_cast<V*>(x)[i];
        V gv = __ldcs(reinterpret_cast<const V*>(g) + i);
        V mv = reinterpret_cast<V*>(m)[i];
        V vv = reinterpret_cast<V*>(v)[i];
        T* xs = reinterpret_cast<T*>(&xv);
        T* gs = reinterpret_cast<T*>(&gv);
        T* ms = reinterpret_cast<T*>(&mv);
        T* vs = reinterpret_cast<T*>(&vv);
#pragma unroll
        for (int k = 0; k < W; ++k) adam1(xs[k], gs[k], ms[k], vs[k], alpha, b1c, b2c, eps);
        reinterpret_cast<V*>(x)[i] = xv;
        reinterpret_cast<V*>(m)[i] = mv;
        reinterpret_cast<V*>(v)[i] = vv;
    }
    for (int64_t i = nv * W + tid; i < n; i += stride) {
        T xs = x[i], ms = m[i], vs = v[i];
        adam1(xs, g[i], ms, vs, alpha, b1c, b2c, eps);
        x[i] = xs;
        m[i] = ms;
        v[i] = vs;
    }
}

// z = a x + b y  (z may alias x or y)
template <typename T>
__global__ void __launch_bounds__(VT) axpby_kernel(T* z, const T* x, const T* y, int64_t n, T a,
                                                   T b, bool vec) {
    using V = typename Vec<T>::V;
    constexpr int W = Vec<T>::W;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nv = vec ? n / W : 0;
    for (int64_t i = tid; i < nv; i += stride) {
        V xv = reinterpret_cast<const V*>(x)[i];
        V yv = reinterpret_cast<const V*>(y)[i];
        T* xs = reinterpret_cast<T*>(&xv);
        const T* ys = reinterpret_cast<const T*>(&yv);
#pragma unroll
        for (int k = 0; k < W; ++k) xs[k] = a * xs[k] + b * ys[k];
        reinterpret_cast<V*>(z)[i] = xv;
    }
    for (int64_t i = nv * W + tid; i < n; i += stride) z[i] = a * x[i] + b * y[i];
}

// ---------------------------------------------------------------------------
// Multi-dot: D[i*r + j] = sum_e M[i*ld + e] * Q_j[e], i < k, j < r <= 4.
// Block (g, c) reduces the MD_G rows g*MD_G ... of M over column chunk c: each
// thread keeps its slice of the r query vectors in registers (read once per
// chunk and row group), streams the group's rows (MD_G independent loads in
// flight), and accumulates MD_G x r partial sums in the working precision.
// The last block adds the chunk partials in index order (deterministic).
constexpr int MD_MAXR = 4;
constexpr int MD_G = 4;

struct QPtrs {
    const void* q[MD_MAXR];
};

template <typename T>
__global__ void __launch_bounds__(VT) multidot_kernel(const T* __restrict__ M, int64_t ld, int k,
                                                      QPtrs qs, int r, int64_t n, int64_t chunk,
                                                      double* __restrict__ partials,
                                                      unsigned* counter, double* __restrict__ out,
                                                      bool vec) {
    using V = typename Vec<T>::V;
    constexpr int W = Vec<T>::W;
    const int g0 = blockIdx.x * MD_G;   // first row of the group
    const int64_t c = blockIdx.y;       // chunk
    const int64_t e0 = c * chunk;
    int64_t e1 = e0 + chunk;
    if (e1 > n) e1 = n;
    T acc[MD_G][MD_MAXR];
#pragma unroll
    for (int g = 0; g < MD_G; ++g)
#pragma unroll
        for (int j = 0; j < MD_MAXR; ++j) acc[g][j] = T(0);
    if (vec) {
        const int64_t v0 = e0 / W, v1 = e1 / W;
        // Two elements per thread and step, all their loads issued before the
        // multiply-adds: 8 row loads in flight per thread.
        auto load = [&](int64_t e, V (&qv)[MD_MAXR], V (&mv)[MD_G]) {
#pragma unroll
            for (int j = 0; j < MD_MAXR; ++j)
                if (j < r) qv[j] = __ldg(reinterpret_cast<const V*>(qs.q[j]) + e);
#pragma unroll
            for (int g = 0; g < MD_G; ++g)
                if (g0 + g < k)
                    mv[g] = __ldcs(reinterpret_cast<const V*>(M + (int64_t)(g0 + g) * ld) + e);
        };
        auto madd = [&](const V (&qv)[MD_MAXR], const V (&mv)[MD_G]) {
#pragma unroll
            for (int g = 0; g < MD_G; ++g) {
                if (g0 + g < k) {
                    const T* ms = reinterpret_cast<const T*>(&mv[g]);
#pragma unroll
                    for (int j = 0; j < MD_MAXR; ++j) {
                        if (j < r) {
                            const T* qq = reinterpret_cast<const T*>(&qv[j]);
#pragma unroll
                            for (int w = 0; w < W; ++w) acc[g][j] += ms[w] * qq[w];
                        }
                    }
                }
            }
        };
        for (int64_t e = v0 + threadIdx.x; e < v1; e += 2 * VT) {
            V qa[MD_MAXR], ma[MD_G], qb[MD_MAXR], mb[MD_G];
            const bool two = e + VT < v1;
            load(e, qa, ma);
            if (two) load(e + VT, qb, mb);
            madd(qa, ma);
            if (two) madd(qb, mb);
        }
        for (int64_t e = v1 * W + threadIdx.x; e < e1; e += VT) {
#pragma unroll
            for (int g = 0; g < MD_G; ++g) {
                if (g0 + g < k) {
                    const T mval = M[(int64_t)(g0 + g) * ld + e];
#pragma unroll
                    for (int j = 0; j < MD_MAXR; ++j)
                        if (j < r) acc[g][j] += mval * ((const T*)qs.q[j])[e];
                }
            }
        }
    } else {
        for (int64_t e = e0 + threadIdx.x; e < e1; e += VT) {
#pragma unroll
            for (int g = 0; g < MD_G; ++g) {
                if (g0 + g < k) {
                    const T mval = M[(int64_t)(g0 + g) * ld + e];
#pragma unroll
                    for (int j = 0; j < MD_MAXR; ++j)
                        if (j < r) acc[g][j] += mval * ((const T*)qs.q[j])[e];
                }
            }
        }
    }
    const int64_t nchunk = gridDim.y;
#pragma unroll
    for (int g = 0; g < MD_G; ++g) {
#pragma unroll
        for (int j = 0; j < MD_MAXR; ++j) {
            if (g0 + g < k && j < r) {
                double s = block_sum((double)acc[g][j]);
                if (threadIdx.x == 0) partials[((int64_t)(g0 + g) * r + j) * nchunk + c] = s;
            }
        }
    }
    if (counter == nullptr) return;  // multidot_finish_kernel adds them
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        is_last = (prev == (unsigned)((int64_t)gridDim.x * gridDim.y - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // Each output's chunk partials summed by the whole block in a fixed order.
    for (int o = 0; o < k * r; ++o) {
        const double s = sum_partials(partials + (int64_t)o * nchunk, nchunk);
        if (threadIdx.x == 0) out[o] = s;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

// Vector path of the multi-dot with the number of vectors R fixed at compile
// time: rows past k in the last group are loaded from row k-1 (valid memory)
// and dropped at the end, so the loop body has no predicate and all 2 (G + R)
// 16-byte loads of two elements per thread are issued before the
// multiply-adds.  Same partial layout and finish as multidot_kernel.
template <typename T, int R, int G>
__global__ void __launch_bounds__(VT, 3) multidot_vec_kernel(
    const T* __restrict__ M, int64_t ld, int k, QPtrs qs, int64_t n, int64_t chunk,
    double* __restrict__ partials, unsigned* counter, double* __restrict__ out) {
    using V = typename Vec<T>::V;
    constexpr int W = Vec<T>::W;
    const int g0 = blockIdx.x * G;
    const int64_t c = blockIdx.y;
    const int64_t e0 = c * chunk;
    int64_t e1 = e0 + chunk;
    if (e1 > n) e1 = n;
    const V* rows[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const int row = g0 + g < k ? g0 + g : k - 1;
        rows[g] = reinterpret_cast<const V*>(M + (int64_t)row * ld);
    }
    const V* qv[R];
#pragma unroll
    for (int j = 0; j < R; ++j) qv[j] = reinterpret_cast<const V*>(qs.q[j]);
    T acc[G][R];
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
        for (int j = 0; j < R; ++j) acc[g][j] = T(0);
    auto madd = [&](const V (&q)[R], const V (&m)[G]) {
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const T* ms = reinterpret_cast<const T*>(&m[g]);
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const T* qq = reinterpret_cast<const T*>(&q[j]);
#pragma unroll
                for (int w = 0; w < W; ++w) acc[g][j] += ms[w] * qq[w];
            }
        }
    };
    // U steps of 16-byte loads per thread issued before their multiply-adds
    // (more steps when the loads per step are few).
    constexpr int U = (R + G) <= 3 ? 4 : 2;
    const int64_t v0 = e0 / W, v1 = e1 / W;
    int64_t e = v0 + threadIdx.x;
    for (; e + (U - 1) * VT < v1; e += U * VT) {
        V q[U][R], m[U][G];
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int j = 0; j < R; ++j) q[u][j] = __ldg(qv[j] + e + u * VT);
#pragma unroll
            for (int g = 0; g < G; ++g) m[u][g] = __ldcs(rows[g] + e + u * VT);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) madd(q[u], m[u]);
    }
    for (; e < v1; e += VT) {
        V qa[R], ma[G];
#pragma unroll
        for (int j = 0; j < R; ++j) qa[j] = __ldg(qv[j] + e);
#pragma unroll
        for (int g = 0; g < G; ++g) ma[g] = __ldcs(rows[g] + e);
        madd(qa, ma);
    }
    for (int64_t t = v1 * W + threadIdx.x; t < e1; t += VT) {  // scalar tail
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const T mval = reinterpret_cast<const T*>(rows[g])[t];
#pragma unroll
            for (int j = 0; j < R; ++j) acc[g][j] += mval * ((const T*)qs.q[j])[t];
        }
    }
    const int64_t nchunk = gridDim.y;
    // All G x R sums in one pass: warp sums, one barrier, then thread o adds
    // the warps' values of sum o in warp order (deterministic).
    __shared__ double red[VT / 32][G * R];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int g = 0; g < G; ++g) {
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const double v = warp_sum((double)acc[g][j]);
            if (lane == 0) red[warp][g * R + j] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < G * R) {
        const int o = threadIdx.x, g = o / R, j = o - g * R;
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < VT / 32; ++w) sum += red[w][o];
        if (g0 + g < k) partials[((int64_t)(g0 + g) * R + j) * nchunk + c] = sum;
        __threadfence();  // each writer publishes its partial device-wide
    }
    if (counter == nullptr) return;  // multidot_finish_kernel adds them
    __shared__ bool is_last;
    __syncthreads();  // every partial of the block is written and fenced
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        is_last = (prev == (unsigned)((int64_t)gridDim.x * gridDim.y - 1));
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // Each output's chunk partials summed by the whole block, 8 loads in
    // flight per thread (fixed order: deterministic).
    for (int o = 0; o < k * R; ++o) {
        const double sum = sum_partials(partials + (int64_t)o * nchunk, nchunk);
        if (threadIdx.x == 0) out[o] = sum;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

// The chunk partials of each of `outputs` results added by one warp per
// result: lane l takes partials l, l + 32, ... and the warp adds the lanes in
// a fixed tree (deterministic).  Used when a multi-dot has more than
// kMdFinishInKernel results, where the last block of the multi-dot would
// otherwise add them one after the other.
constexpr int kMdFinishInKernel = 8;

__global__ void __launch_bounds__(256) multidot_finish_kernel(const double* __restrict__ partials,
                                                              int64_t nchunk, int64_t outputs,
                                                              double* __restrict__ out) {
    const int64_t o = ((int64_t)blockIdx.x * 256 + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (o >= outputs) return;
    const double* p = partials + o * nchunk;
    double s = 0.0;
    for (int64_t c = lane; c < nchunk; c += 32) s += __ldcg(p + c);
    s = warp_sum(s);
    if (lane == 0) out[o] = s;
}

// out = c0 * x + sum_i coef[i] * M_i  (coef, c0 read from device memory);
// with dot given, also dot[0] = <out, x> (per-thread sums in the working
// precision, FP64 across blocks, added in index order by the last block).
template <typename T>
__global__ void __launch_bounds__(VT) lincomb_kernel(T* __restrict__ out, const T* __restrict__ x,
                                                     const T* __restrict__ M, int64_t ld, int k,
                                                     const double* __restrict__ coef,
                                                     int64_t n, bool vec, ReduceWs ws,
                                                     double* __restrict__ dot) {
    using V = typename Vec<T>::V;
    constexpr int W = Vec<T>::W;
    __shared__ T sc[257];
    for (int i = threadIdx.x; i <= k; i += blockDim.x) sc[i] = (T)coef[i];
    __syncthreads();
    const T c0 = sc[k];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nv = vec ? n / W : 0;
    T dsum = T(0);
    for (int64_t e = tid; e < nv; e += stride) {
        const V x0 = __ldcs(reinterpret_cast<const V*>(x) + e);
        V xv = x0;
        T* acc = reinterpret_cast<T*>(&xv);
#pragma unroll
        for (int w = 0; w < W; ++w) acc[w] *= c0;
        for (int i = 0; i < k; ++i) {
            V mv = __ldcs(reinterpret_cast<const V*>(M + (int64_t)i * ld) + e);
            const T* ms = reinterpret_cast<const T*>(&mv);
            const T ci = sc[i];
#pragma unroll
            for (int w = 0; w < W; ++w) acc[w] += ci * ms[w];
        }
        reinterpret_cast<V*>(out)[e] = xv;
        const T* xs = reinterpret_cast<const T*>(&x0);
#pragma unroll
        for (int w = 0; w < W; ++w) dsum += acc[w] * xs[w];
    }
    for (int64_t e = nv * W + tid; e < n; e += stride) {
        const T xe = x[e];
        T acc = c0 * xe;
        for (int i = 0; i < k; ++i) acc += sc[i] * M[(int64_t)i * ld + e];
        out[e] = acc;
        dsum += acc * xe;
    }
    if (dot) reduce_finish((double)dsum, blockIdx.x, gridDim.x, ws, 1.0, dot);
}

template <typename T>
int adam_impl(T* x, const T* g, T* m, T* v, int64_t n, double alpha, double beta1, double beta2,
              double eps, void* stream) {
    if (n < 0) return ODIL_ERR_SHAPE;
    if (n == 0) return ODIL_OK;
    if (!x || !g || !m || !v) return ODIL_ERR_ARG;
    const bool vec = aligned16(x) && aligned16(g) && aligned16(m) && aligned16(v);
    const int blocks = stream_blocks(n, Vec<T>::W);
    adam_kernel<T><<<blocks, VT, 0, as_stream(stream)>>>(x, g, m, v, n, (T)alpha,
                                                         (T)(1.0 - beta1), (T)(1.0 - beta2),
                                                         (T)eps, vec);
    return launch_status();
}

template <typename T>
int axpby_impl(T* z, const T* x, const T* y, int64_t n, double a, double b, void* stream) {
    if (n < 0) return ODIL_ERR_SHAPE;
    if (n == 0) return ODIL_OK;
    if (!z || !x || !y) return ODIL_ERR_ARG;
    const bool vec = aligned16(z) && aligned16(x) && aligned16(y);
    axpby_kernel<T><<<stream_blocks(n, Vec<T>::W), VT, 0, as_stream(stream)>>>(z, x, y, n, (T)a,
                                                                               (T)b, vec);
    return launch_status();
}

// Chunk length: about kMdBlocks blocks in all (152 SMs x 3 resident blocks:
// one wave of long-running blocks, so no tail wave and the per-block
// reduction is paid once per block), chunks a multiple of 1024 elements and
// at least 4096.
constexpr int64_t kMdBlocks = 152 * 3;

inline int64_t md_chunk(int64_t n, int k) {
    const int64_t groups = (k + MD_G - 1) / MD_G;
    int64_t per = kMdBlocks / groups;
    if (per < 1) per = 1;
    int64_t chunk = ((n + per - 1) / per + 1023) / 1024 * 1024;
    if (chunk < 4096) chunk = 4096;
    return chunk;
}

// Workspace one call with k rows and r vectors needs.
inline int64_t md_ws_need(int64_t n, int k, int r) {
    const int64_t nchunk = (n + md_chunk(n, k) - 1) / md_chunk(n, k);
    return kReduceHeader + (int64_t)k * r * nchunk * (int64_t)sizeof(double);
}

// Workspace that serves every call with at most k rows and r vectors (fewer
// rows can mean more chunks, so the need is not monotone in k; its maximum
// sits at a row count that fills its last group).
inline int64_t md_ws_bytes(int64_t n, int k, int r) {
    int64_t most = 0;
    for (int64_t groups = 1; (groups - 1) * MD_G < k; ++groups) {
        const int rows = (int)(groups * MD_G < k ? groups * MD_G : k);
        const int64_t need = md_ws_need(n, rows, r);
        if (need > most) most = need;
    }
    return most;
}

template <typename T, int G>
int md_vec_launch(dim3 grid, cudaStream_t st, const T* M, int64_t ld, int k, QPtrs qs, int r,
                  int64_t n, int64_t chunk, ReduceWs w, double* out) {
    switch (r) {
        case 1:
            multidot_vec_kernel<T, 1, G><<<grid, VT, 0, st>>>(M, ld, k, qs, n, chunk, w.partials,
                                                               w.counter, out);
            break;
        case 2:
            multidot_vec_kernel<T, 2, G><<<grid, VT, 0, st>>>(M, ld, k, qs, n, chunk, w.partials,
                                                               w.counter, out);
            break;
        case 3:
            multidot_vec_kernel<T, 3, G><<<grid, VT, 0, st>>>(M, ld, k, qs, n, chunk, w.partials,
                                                               w.counter, out);
            break;
        default:
            multidot_vec_kernel<T, 4, G><<<grid, VT, 0, st>>>(M, ld, k, qs, n, chunk, w.partials,
                                                               w.counter, out);
            break;
    }
    return launch_status();
}

template <typename T>
int multidot_impl(const T* M, int64_t ld, int k, const void* const* q, int r, int64_t n,
                  double* out, void* ws, int64_t ws_bytes, void* stream) {
    if (k < 1 || r < 1 || r > MD_MAXR || n < 1 || ld < n || k > 65535) return ODIL_ERR_SHAPE;
    if (!M || !q || !out) return ODIL_ERR_ARG;
    if (!ws || ws_bytes < md_ws_need(n, k, r)) return ODIL_ERR_WORKSPACE;
    QPtrs qs = {};
    bool vec = aligned16(M) && ((ld * (int64_t)sizeof(T)) % 16 == 0);
    for (int j = 0; j < r; ++j) {
        if (!q[j]) return ODIL_ERR_ARG;
        qs.q[j] = q[j];
        vec = vec && aligned16(q[j]);
    }
    const int64_t chunk = md_chunk(n, k);
    const int64_t nchunk = (n + chunk - 1) / chunk;
    if (nchunk > 65535) return ODIL_ERR_SHAPE;
    ReduceWs w = reduce_ws(ws);
    dim3 grid((k + MD_G - 1) / MD_G, (unsigned)nchunk);
    cudaStream_t st = as_stream(stream);
    // Many results: the multi-dot only writes partials, a second launch adds
    // them in parallel; few: its last block adds them.
    const int64_t outputs = (int64_t)k * r;
    const bool sep = outputs > kMdFinishInKernel;
    if (sep) w.counter = nullptr;
    int rc;
    if (vec) {
        // Row groups of G = min(k, 4) rows (k = 3 loads row 2 twice).
        if (k == 1) rc = md_vec_launch<T, 1>(grid, st, M, ld, k, qs, r, n, chunk, w, out);
        else if (k == 2) rc = md_vec_launch<T, 2>(grid, st, M, ld, k, qs, r, n, chunk, w, out);
        else rc = md_vec_launch<T, MD_G>(grid, st, M, ld, k, qs, r, n, chunk, w, out);
    } else {
        multidot_kernel<T><<<grid, VT, 0, st>>>(M, ld, k, qs, r, n, chunk, w.partials, w.counter,
                                                out, vec);
        rc = launch_status();
    }
    if (rc || !sep) return rc;
    multidot_finish_kernel<<<(unsigned)((outputs * 32 + 255) / 256), 256, 0, st>>>(
        w.partials, nchunk, outputs, out);
    return launch_status();
}

template <typename T>
int lincomb_impl(T* out, const T* x, const T* M, int64_t ld, int k, const double* coef, int64_t n,
                 double* dot, void* ws, int64_t ws_bytes, void* stream) {
    if (k < 0 || k > 256 || n < 1 || (k > 0 && ld < n)) return ODIL_ERR_SHAPE;
    if (!out || !x || !coef || (k > 0 && !M)) return ODIL_ERR_ARG;
    const bool vec = aligned16(out) && aligned16(x) && (k == 0 || (aligned16(M) &&
                                                                  (ld * (int64_t)sizeof(T)) % 16 == 0));
    const int blocks = stream_blocks(n, Vec<T>::W);
    ReduceWs w{nullptr, nullptr};
    if (dot) {
        if (!ws || ws_bytes < reduce_ws_bytes(blocks)) return ODIL_ERR_WORKSPACE;
        w = reduce_ws(ws);
    }
    lincomb_kernel<T><<<blocks, VT, 0, as_stream(stream)>>>(out, x, M, ld, k, coef, n, vec, w,
                                                            dot);
    return launch_status();
}

// out = hi + lo in FP64 (lo may be null), exactly (the sum of two floats
// with exponents at most 28 apart fits in a double): integer instructions
// only in that common case, the FP64 add otherwise.
__global__ void __launch_bounds__(VT) pair_to_f64_kernel(const float* __restrict__ hi,
                                                         const float* __restrict__ lo,
                                                         double* __restrict__ out, int64_t n,
                                                         bool vec) {
    pdl_trigger();
    pdl_wait();  // hi / lo come from the kernel before (PDL launch)
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (vec) {  // 4 elements per thread: 16-byte loads, two 16-byte stores
        for (int64_t v = t0; v < n / 4; v += stride) {
            const float4 h = __ldcs(reinterpret_cast<const float4*>(hi) + v);
            float4 l = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lo) l = __ldcs(reinterpret_cast<const float4*>(lo) + v);
            double2 a, c;
            if (lo) {
                a.x = pair_sum_exact(h.x, l.x);
                a.y = pair_sum_exact(h.y, l.y);
                c.x = pair_sum_exact(h.z, l.z);
                c.y = pair_sum_exact(h.w, l.w);
            } else {
                a.x = f2d_exact(h.x);
                a.y = f2d_exact(h.y);
                c.x = f2d_exact(h.z);
                c.y = f2d_exact(h.w);
            }
            __stcs(reinterpret_cast<double2*>(out) + 2 * v, a);
            __stcs(reinterpret_cast<double2*>(out) + 2 * v + 1, c);
        }
        for (int64_t i = n / 4 * 4 + t0; i < n; i += stride) {
            double v = f2d_exact(__ldcs(hi + i));
            if (lo) v += f2d_exact(__ldcs(lo + i));
            out[i] = v;
        }
        return;
    }
    for (int64_t i = t0; i < n; i += stride) {
        double v = f2d_exact(__ldcs(hi + i));
        if (lo) v += f2d_exact(__ldcs(lo + i));
        out[i] = v;
    }
}

// out = u + (double)d: the FP64 update of a mixed-precision step.
__global__ void __launch_bounds__(VT) add_f32_to_f64_kernel(const double* __restrict__ u,
                                                            const float* __restrict__ d,
                                                            double* __restrict__ out, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = __ldcs(u + i) + f2d_exact(__ldcs(d + i));
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_adam_step_f32(float* x, const float* g, float* m, float* v, int64_t n,
                                double alpha, double beta1, double beta2, double epsilon,
                                void* stream) {
    return adam_impl<float>(x, g, m, v, n, alpha, beta1, beta2, epsilon, stream);
}
ODIL_API int odil_adam_step_f64(double* x, const double* g, double* m, double* v, int64_t n,
                                double alpha, double beta1, double beta2, double epsilon,
                                void* stream) {
    return adam_impl<double>(x, g, m, v, n, alpha, beta1, beta2, epsilon, stream);
}
ODIL_API int odil_axpby_f32(float* z, const float* x, const float* y, int64_t n, double a,
                            double b, void* stream) {
    return axpby_impl<float>(z, x, y, n, a, b, stream);
}
ODIL_API int odil_axpby_f64(double* z, const double* x, const double* y, int64_t n, double a,
                            double b, void* stream) {
    return axpby_impl<double>(z, x, y, n, a, b, stream);
}
ODIL_API int64_t odil_multidot_workspace_bytes(int64_t n, int k, int r) {
    if (n < 1 || k < 1 || r < 1) return 0;
    return md_ws_bytes(n, k, r);
}
ODIL_API int odil_multidot_f32(const float* M, int64_t ld, int k, const void* const* q, int r,
                               int64_t n, double* out, void* workspace, int64_t workspace_bytes,
                               void* stream) {
    return multidot_impl<float>(M, ld, k, q, r, n, out, workspace, workspace_bytes, stream);
}
ODIL_API int odil_multidot_f64(const double* M, int64_t ld, int k, const void* const* q, int r,
                               int64_t n, double* out, void* workspace, int64_t workspace_bytes,
                               void* stream) {
    return multidot_impl<double>(M, ld, k, q, r, n, out, workspace, workspace_bytes, stream);
}
ODIL_API int odil_lincomb_f32(float* out, const float* x, const float* M, int64_t ld, int k,
                              const double* coef, int64_t n, void* stream) {
    return lincomb_impl<float>(out, x, M, ld, k, coef, n, nullptr, nullptr, 0, stream);
}
ODIL_API int odil_lincomb_f64(double* out, const double* x, const double* M, int64_t ld, int k,
                              const double* coef, int64_t n, void* stream) {
    return lincomb_impl<double>(out, x, M, ld, k, coef, n, nullptr, nullptr, 0, stream);
}

ODIL_API int64_t odil_lincomb_dot_workspace_bytes(int64_t n) {
    if (n < 1) return 0;
    const int a = stream_blocks(n, Vec<float>::W), b = stream_blocks(n, Vec<double>::W);
    return reduce_ws_bytes(a > b ? a : b);
}
ODIL_API int odil_lincomb_dot_f32(float* out, const float* x, const float* M, int64_t ld, int k,
                                  const double* coef, int64_t n, double* dot, void* workspace,
                                  int64_t workspace_bytes, void* stream) {
    if (!dot) return ODIL_ERR_ARG;
    return lincomb_impl<float>(out, x, M, ld, k, coef, n, dot, workspace, workspace_bytes, stream);
}
ODIL_API int odil_lincomb_dot_f64(double* out, const double* x, const double* M, int64_t ld,
                                  int k, const double* coef, int64_t n, double* dot,
                                  void* workspace, int64_t workspace_bytes, void* stream) {
    if (!dot) return ODIL_ERR_ARG;
    return lincomb_impl<double>(out, x, M, ld, k, coef, n, dot, workspace, workspace_bytes,
                                stream);
}

ODIL_API int odil_add_f32_to_f64(const double* u, const float* d, double* out, int64_t n,
                                 void* stream) {
    if (n < 0) return ODIL_ERR_SHAPE;
    if (n == 0) return ODIL_OK;
    if (!u || !d || !out) return ODIL_ERR_ARG;
    add_f32_to_f64_kernel<<<stream_blocks(n, 1), VT, 0, as_stream(stream)>>>(u, d, out, n);
    return launch_status();
}

ODIL_API int odil_pair_to_f64(const float* hi, const float* lo, double* out, int64_t n,
                              void* stream) {
    if (n < 0) return ODIL_ERR_SHAPE;
    if (n == 0) return ODIL_OK;
    if (!hi || !out) return ODIL_ERR_ARG;
    const bool vec = aligned16(hi) && aligned16(out) && (!lo || aligned16(lo));
    if (launch_pdl(pair_to_f64_kernel, dim3(stream_blocks(n, vec ? 4 : 1)), dim3(VT), 0,
                   as_stream(stream), hi, lo, out, n, vec) != cudaSuccess)
        return launch_status();
    return launch_status();
}
