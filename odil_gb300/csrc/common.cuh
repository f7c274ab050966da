// Shared device helpers of libodil_gb300: status handling, index wrapping and
// the deterministic two-level FP64 reduction used by every loss kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/odil_gb300.h"

#define ODIL_API extern "C" __attribute__((visibility("default")))

namespace odil {

inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ODIL_OK : ODIL_ERR_LAUNCH;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Raises a kernel's dynamic shared-memory limit the first time a launch needs
// more than 48 KiB (per kernel, keyed by its address), so later launches --
// including those recorded into CUDA graphs -- make no attribute calls.
inline void ensure_dynamic_smem(const void* kern, size_t bytes) {
    constexpr int kSlots = 64;
    static const void* keys[kSlots];
    static size_t vals[kSlots];
    static int used = 0;
    if (bytes <= 48 * 1024) return;
    for (int i = 0; i < used; ++i) {
        if (keys[i] == kern) {
            if (vals[i] >= bytes) return;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            vals[i] = bytes;
            return;
        }
    }
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (used < kSlots) {
        keys[used] = kern;
        vals[used] = bytes;
        ++used;
    }
}

// Exact FP32 -> FP64 conversion with integer instructions (normal numbers,
// zeros, infinities, NaN; subnormal inputs take the hardware conversion).
__device__ __forceinline__ double f2d_exact(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u && (b & 0x7fffffu) != 0u) return (double)x;
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    const unsigned long long mant = (unsigned long long)(b & 0x7fffffu) << 29;
    unsigned long long de;
    if (e == 0u) de = 0ull;
    else if (e == 0xffu) de = 0x7ffull;
    else de = (unsigned long long)(e + (1023u - 127u));
    return __longlong_as_double((long long)(sign | (de << 52) | mant));
}

// (double)h + (double)l, exactly when the sum fits in a double, with integer
// instructions only in the common case: both normal, exponents at most 28
// apart, so the aligned integer sum has at most 53 significant bits and is
// exact.  Other cases (zeros, subnormals, wide gaps) take the FP64 add, which
// is exact or correctly rounded the same way.
__device__ __forceinline__ double pair_sum_exact(float h, float l) {
    unsigned bh = __float_as_uint(h), bl = __float_as_uint(l);
    unsigned eh = (bh >> 23) & 0xffu, el = (bl >> 23) & 0xffu;
    if (eh < el) {
        const unsigned t = bh; bh = bl; bl = t;
        const unsigned te = eh; eh = el; el = te;
    }
    const unsigned d = eh - el;
    if (el == 0u || eh == 0xffu || d > 28u) return f2d_exact(h) + f2d_exact(l);
    const long long mh = (long long)((bh & 0x7fffffu) | 0x800000u);
    const long long ml = (long long)((bl & 0x7fffffu) | 0x800000u);
    long long M = mh << d;
    M = ((bh ^ bl) >> 31) ? M - ml : M + ml;  // magnitude of |big| -+ |small|
    if (M == 0) return 0.0;
    unsigned long long sign = (unsigned long long)(bh >> 31) << 63;
    if (M < 0) {  // equal exponents, |small| > |big|: the small one's sign
        M = -M;
        sign ^= 1ull << 63;
    }
    const int p = 63 - __clzll(M);  // top bit, p <= 52
    const unsigned long long mant =
        ((unsigned long long)M << (52 - p)) & ((1ull << 52) - 1ull);
    const unsigned long long ex = (unsigned long long)(p + (int)el - 150 + 1023);
    return __longlong_as_double((long long)(sign | (ex << 52) | mant));
}

// Periodic wrap of an index that is at most one period outside [0, n).
__device__ __forceinline__ int wrap1(int i, int n) {
    return i < 0 ? i + n : (i >= n ? i - n : i);
}
// Periodic wrap of an arbitrary index.
__device__ __forceinline__ int wrapn(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block; the result is valid in every thread.  Fixed tree, so
// the result is bitwise reproducible for a fixed blockDim.
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double red[32];
    __shared__ double total;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarp = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();  // protect `red` and `total` against a previous call
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double w = lane < nwarp ? red[lane] : 0.0;
        w = warp_sum(w);
        if (lane == 0) total = w;
    }
    __syncthreads();
    return total;
}

// Workspace layout of a reduction: [counter | pad to 256 B | partials...].
struct ReduceWs {
    unsigned* counter;
    double* partials;
};

constexpr int64_t kReduceHeader = 256;

inline int64_t reduce_ws_bytes(int64_t nblocks) {
    return kReduceHeader + nblocks * (int64_t)sizeof(double);
}

inline ReduceWs reduce_ws(void* ws) {
    ReduceWs r;
    r.counter = reinterpret_cast<unsigned*>(ws);
    r.partials = reinterpret_cast<double*>(reinterpret_cast<char*>(ws) + kReduceHeader);
    return r;
}

// Sum of partials[0 .. count) by the whole block in a fixed order (bitwise
// reproducible for a fixed blockDim): each thread keeps 8 loads in flight, so
// a single warp finishing thousands of partial sums is not bound by one L2
// round trip per partial.
__device__ __forceinline__ double sum_partials(const double* partials, int64_t count) {
    constexpr int U = 8;
    double acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc[u] = 0.0;
    const int64_t step = (int64_t)blockDim.x * U;
    for (int64_t k0 = threadIdx.x; k0 < count; k0 += step) {
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t k = k0 + (int64_t)u * blockDim.x;
            v[u] = k < count ? __ldcg(partials + k) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc[u] += v[u];
    }
    double s = 0.0;
#pragma unroll
    for (int u = 0; u < U; ++u) s += acc[u];
    return block_sum(s);
}

// Called by every thread of every block with the thread's partial sum.  Block
// `bid` of `nblocks` stores its sum; the last block to arrive adds the partial
// sums in index order (deterministic), writes out[0] = sum * scale and resets
// the counter to zero for the next call.
__device__ __forceinline__ void reduce_finish(double v, int64_t bid, int64_t nblocks,
                                              ReduceWs ws, double scale, double* out) {
    __shared__ bool is_last;
    v = block_sum(v);
    if (threadIdx.x == 0) {
        ws.partials[bid] = v;
        __threadfence();
        unsigned prev = atomicAdd(ws.counter, 1u);
        is_last = (prev == (unsigned)(nblocks - 1));
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        double s = sum_partials(ws.partials, nblocks);
        if (threadIdx.x == 0) {
            out[0] = s * scale;
            *ws.counter = 0u;
        }
    }
}

// Programmatic dependent launch.  pdl_trigger: this grid's dependents may
// launch now (they still wait for its completion before reading its
// output).  pdl_wait: wait until the grids this one depends on have
// completed and their writes are visible (returns at once when the launch
// had no programmatic dependency).
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

// Launches `kern` on `st` with programmatic stream serialisation allowed, so
// that it may start while the previous kernel in the stream finishes (it
// must call pdl_wait before touching that kernel's output).
template <typename... Args>
cudaError_t launch_pdl(void (*kern)(Args...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace odil
