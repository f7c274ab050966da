// Forward substitution along t for the wave Jacobian (the direct solve that
// linsolver.py:35-45 does with SuperLU), spread over a thread-block cluster.
//
// Row i of the solution depends on row i-1 at columns j-1, j, j+1 and on row
// i-2 at column j only, so a column range known at rows i-1 and i-2 on a
// window H columns wider on each side determines the range itself for H more
// rows.  Each warp owns O = 32 CPT - 2H columns and marches a 32 CPT-column
// window (its own columns plus H halo columns on each side) for H rows with
// no communication but register shuffles; the halo values it computes go
// stale from the window's edges inwards, one column per row, and never reach
// the owned columns.  Every H rows the cluster synchronises (release/acquire)
// and each warp reloads its halo columns of the last two rows from the
// solution its neighbours stored.  One warp per SM sub-partition runs a
// dependent chain of a few FMAs and two shuffles per row, instead of one
// block-wide barrier per row on a single SM.
//
// The arithmetic per cell is that of the single-block march (wave_dev.cuh),
// with the column-class factors k_tm, k_xm, k_xp of the boundary closure.

#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "wave_dev.cuh"

namespace odil {
namespace {

using wavedev::k_tm;
using wavedev::k_xm;
using wavedev::k_xp;
using wavedev::make_dev;
using wavedev::WaveDev;

constexpr int kTiledMaxWarps = 4;  // warps (tiles) per block: one per SM sub-partition

// A lane's CPT contiguous columns as 16-byte (or 8-byte) vector accesses,
// element by element into registers.
template <typename T, int CPT>
__device__ __forceinline__ void ld_cols(T (&o)[CPT], const T* __restrict__ p) {
    if constexpr (sizeof(T) == 4 && CPT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 4; ++q) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(p) + q);
            o[4 * q] = v.x;
            o[4 * q + 1] = v.y;
            o[4 * q + 2] = v.z;
            o[4 * q + 3] = v.w;
        }
    } else if constexpr (sizeof(T) == 4 && CPT == 2) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        o[0] = v.x;
        o[1] = v.y;
    } else if constexpr (sizeof(T) == 8 && CPT % 2 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 2; ++q) {
            const double2 v = __ldg(reinterpret_cast<const double2*>(p) + q);
            o[2 * q] = v.x;
            o[2 * q + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int c = 0; c < CPT; ++c) o[c] = __ldg(p + c);
    }
}

template <typename T, int CPT>
__device__ __forceinline__ void st_cols(T* p, const T (&v)[CPT]) {
    if constexpr (sizeof(T) == 4 && CPT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 4; ++q)
            reinterpret_cast<float4*>(p)[q] =
                make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else if constexpr (sizeof(T) == 4 && CPT == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else if constexpr (sizeof(T) == 8 && CPT % 2 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 2; ++q)
            reinterpret_cast<double2*>(p)[q] = make_double2(v[2 * q], v[2 * q + 1]);
    } else {
#pragma unroll
        for (int c = 0; c < CPT; ++c) p[c] = v[c];
    }
}

// ---- distributed shared memory exchange --------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_map(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes)
                 : "memory");
}

// Non-blocking test of the phase with the given parity (the caller spins:
// the wait is short and a suspended warp would wake late).
__device__ __forceinline__ bool mbar_test_wait(uint32_t mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;\n" : "=l"(t));
    return t;
}

// Stores CPT values into another CTA's shared memory; the bytes count
// towards that CTA's mbarrier transaction (st.async, no fence needed).
template <typename T, int CPT>
__device__ __forceinline__ void push_cols(uint32_t raddr, uint32_t rmbar, const T (&v)[CPT]) {
    if constexpr (sizeof(T) == 4 && CPT % 4 == 0) {
#pragma unroll
        for (int q = 0; q < CPT / 4; ++q)
            asm volatile(
                "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, "
                "[%5];\n" ::"r"(raddr + 16 * q),
                "f"(v[4 * q]), "f"(v[4 * q + 1]), "f"(v[4 * q + 2]), "f"(v[4 * q + 3]), "r"(rmbar)
                : "memory");
    } else if constexpr (sizeof(T) == 4 && CPT == 2) {
        asm volatile(
            "st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];\n" ::"r"(
                raddr),
            "f"(v[0]), "f"(v[1]), "r"(rmbar)
            : "memory");
    } else {
        static_assert(sizeof(T) == 8 && CPT % 2 == 0, "pushed run");
#pragma unroll
        for (int q = 0; q < CPT / 2; ++q)
            asm volatile(
                "st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, "
                "[%3];\n" ::"r"(raddr + 16 * q),
                "d"(v[2 * q]), "d"(v[2 * q + 1]), "r"(rmbar)
                : "memory");
    }
}

// A halo wait that gives up after this long (the whole march takes well under
// a millisecond); the warp then writes NaN and counts the failure.
constexpr uint64_t kHaloWaitNs = 1000000000ull;
__device__ unsigned long long g_tiled_wait_failures = 0;

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// VEC: nx % CPT == 0 and b, x aligned to CPT elements (capped at 16 bytes),
// so a lane's columns are all inside the row or all outside it and its loads
// and stores are whole vector accesses.
// PF right-hand-side rows are in flight per lane (a register ring): the loads
// of row i+PF-1 are issued while row i is computed.
//
// Columns outside the row carry zero factors, a zero right-hand side and zero
// start values, so they stay exactly zero with no masking (their neighbours
// only ever meet them multiplied by zero factors, and stay finite).
//
// DSMEM (requires O >= H): instead of a cluster barrier and a reload from
// global memory, at the end of a batch the lanes holding a warp's first and
// last H owned columns push rows i0-2 and i0-1 of them into the halo buffers
// of the neighbouring warps' shared memory with st.async; each warp waits for
// its halo bytes on an mbarrier (double-buffered by batch parity).  Warps
// only wait for their neighbours, and the solution stores need no fence.
// `extra_wait` adds bytes that never arrive to every wait (a planted
// failure for the bounded-wait test; 0 otherwise).
// TBL (march from u = 0): b is the boundary table of -F(0) in the bnd_cell
// order (rows 0 and 1, then columns 0 and nx-1 of each further row); the
// right-hand side is zero elsewhere, so rows 2.. load only the two edge
// entries (the lanes holding columns 0 and nx-1) and the full right-hand
// side is never written or read.
template <typename T, int CPT, int H, int PF, bool VEC, bool DSMEM, bool TBL = false>
__global__ void __launch_bounds__(32 * kTiledMaxWarps) wave_march_tiled_kernel(
    WaveDev<T> g, const T* __restrict__ b, T* __restrict__ x, uint32_t extra_wait) {
    constexpr int O = 32 * CPT - 2 * H;  // owned columns per warp
    static_assert(O > 0 && H % CPT == 0 && H % PF == 0, "tile shape");
    static_assert(!DSMEM || O >= H, "pushed columns come from one neighbour");
    const int nx = g.nx, nt = g.nt;
    const int lane = threadIdx.x & 31;
    const int tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int j0 = tile * O - H + lane * CPT;  // this lane's first column
    const bool own = lane >= H / CPT && lane < (H + O) / CPT;
    bool in[CPT];
    T km[CPT], kt[CPT], kp[CPT], d1[CPT], d2[CPT];
    bool any_in = false;
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
        const int j = j0 + c;
        in[c] = j >= 0 && j < nx;
        any_in |= in[c];
        kt[c] = in[c] ? k_tm<T>(j, nx) : T(0);
        km[c] = in[c] ? k_xm<T>(j, nx) : T(0);
        kp[c] = in[c] ? k_xp<T>(j, nx) : T(0);
        d1[c] = T(0);
        d2[c] = T(0);
    }
    const bool st_ok = own && any_in;
    bool bad = false;  // a halo wait gave up: outputs are NaN from then on
    const T lam = g.lam2, dt2 = g.dt2;
    T pre[PF][CPT];
#pragma unroll
    for (int q = 0; q < PF; ++q)
#pragma unroll
        for (int c = 0; c < CPT; ++c) pre[q][c] = T(0);
    // Launched with programmatic serialisation: the right-hand side is the
    // previous kernel's output.
    pdl_trigger();
    pdl_wait();
    const T* src = b + j0;  // row `next` of the right-hand side
    int next = 0;
    // TBL: the lane's column-table entry of row `next` (entries 2 (r - 2)
    // and 2 (r - 2) + 1 hold columns 0 and nx - 1 of row r >= 2; nx >= 2),
    // for the lane holding that column, and which of its columns it is.
    bool e_b[CPT];
    int toff = 0;
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
        e_b[c] = TBL && (j0 + c == 0 || j0 + c == nx - 1);
        if (TBL && j0 + c == nx - 1) toff = 1;
    }
    const T* tcol = b + 2 * (int64_t)nx + toff;
    // HEAD: the prefetch before the first row (rows 0 .. PF - 2, which hold
    // rows 0 and 1); every later issue is of a row >= PF - 1 >= 2, so with
    // TBL it takes only the table-entry path (no branch in the row bodies).
    static_assert(PF >= 3, "rows 0 and 1 are prefetched ahead of the march");
    auto issue = [&](auto checked, int slot, auto head) {
        constexpr bool HEAD = decltype(head)::value;
        if (!decltype(checked)::value || next < nt) {
            if (!TBL || (HEAD && next < 2)) {
                if constexpr (VEC) {
                    if (any_in) ld_cols<T, CPT>(pre[slot], src);
                } else {
#pragma unroll
                    for (int c = 0; c < CPT; ++c) pre[slot][c] = in[c] ? __ldg(src + c) : T(0);
                }
            } else {
                // Every lane loads (one or two addresses per warp, no
                // divergence); only the boundary column keeps the value.
                const T v = __ldg(tcol);
#pragma unroll
                for (int c = 0; c < CPT; ++c) pre[slot][c] = e_b[c] ? v : T(0);
                tcol += 2;
            }
        }
        src += nx;
        ++next;
    };
#pragma unroll
    for (int q = 0; q < PF - 1; ++q) issue(std::true_type{}, q, std::true_type{});
    T* dst = x + j0;  // solution row i
    // One row: FIRST for rows 0 and 1 of J (identity row; no u[i-2] term),
    // CHECKED where the prefetch may pass the last row.
    auto row = [&](auto first, auto checked, int i, int s) {
        constexpr bool FIRST = decltype(first)::value;
        issue(checked, (s + PF - 1) % PF, std::false_type{});
        const T c_rhs = FIRST && i == 0 ? T(1) : dt2;
        const T c_d1 = FIRST && i == 1 ? T(1) : T(2);
        const T c_lam = FIRST && i == 0 ? T(0) : lam;
        // At the window's ends the shuffles return the lane's own value:
        // finite, and it only feeds stale halo or out-of-row columns.
        const T left = __shfl_up_sync(0xffffffffu, d1[CPT - 1], 1);
        const T right = __shfl_down_sync(0xffffffffu, d1[0], 1);
        T out[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const T xm = c == 0 ? left : d1[c - 1];
            const T xp = c == CPT - 1 ? right : d1[c + 1];
            // The second difference first, then scaled: the rounding of the
            // single-block march (folding lam into the factors loses accuracy
            // to cancellation).
            const T tprev = c_d1 * d1[c] - d2[c];
            out[c] = c_rhs * pre[s][c] + tprev + c_lam * (km[c] * xm - kt[c] * d1[c] + kp[c] * xp);
        }
        if (DSMEM && bad) {
#pragma unroll
            for (int c = 0; c < CPT; ++c) out[c] = T(NAN);
        }
        if (st_ok) {
            if constexpr (VEC) {
                st_cols<T, CPT>(dst, out);
            } else {
#pragma unroll
                for (int c = 0; c < CPT; ++c)
                    if (in[c]) dst[c] = out[c];
            }
        }
        dst += nx;
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            d2[c] = d1[c];
            d1[c] = out[c];
        }
    };
    // DSMEM exchange state: [warp][parity][side 0 left / 1 right][row 0: i0-2,
    // 1: i0-1][H] halo values, one mbarrier per warp and parity.
    __shared__ __align__(16) T halo[DSMEM ? kTiledMaxWarps : 1][2][2][2][DSMEM ? H : 1];
    __shared__ __align__(8) uint64_t mbar[DSMEM ? kTiledMaxWarps : 1][2];
    const int warp = threadIdx.x >> 5;
    const int ntiles = (nx + O - 1) / O;
    const bool active = tile < ntiles;
    const bool has_l = tile >= 1 && active, has_r = tile + 1 < ntiles;
    uint32_t push_addr = 0, push_mbar = 0;  // this lane's push target
    if constexpr (DSMEM) {
        if (lane == 0) {
            mbar_init(smem_u32(&mbar[warp][0]), 1);
            mbar_init(smem_u32(&mbar[warp][1]), 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        // Lanes of the first H owned columns feed the left neighbour's right
        // halo; lanes of the last H owned columns the right neighbour's left.
        const int wl = lane * CPT;  // window column of this lane
        int target = -1, side = 0, off = 0;
        if (has_l && wl >= H && wl < 2 * H) {
            target = tile - 1, side = 1, off = wl - H;
        } else if (has_r && wl >= O && wl < O + H) {
            target = tile + 1, side = 0, off = wl - O;
        }
        if (target >= 0) {
            const int wpb = blockDim.x >> 5;
            const uint32_t rank = (uint32_t)(target / wpb), tw = (uint32_t)(target % wpb);
            push_addr = cluster_map(smem_u32(&halo[tw][0][side][0][off]), rank);
            push_mbar = cluster_map(smem_u32(&mbar[tw][0]), rank);
        }
    }
    if constexpr (DSMEM) cluster_sync_all();  // mbarriers initialised everywhere
    const uint32_t halo_bytes = (has_l ? 1u : 0u) * 2 * H * sizeof(T) +
                                (has_r ? 1u : 0u) * 2 * H * sizeof(T) + extra_wait;
    // Byte offset between the parity-1 and parity-0 copies of halo / mbar.
    constexpr uint32_t kHaloPar = 2 * 2 * (DSMEM ? H : 1) * sizeof(T);
    for (int i0 = 0; i0 < nt && (!DSMEM || active); i0 += H) {
        if (i0 > 0) {
            if constexpr (DSMEM) {
                const int k = i0 / H;
                const int par = k & 1;
                if (halo_bytes > 0 && !bad) {
                    const uint32_t mb = smem_u32(&mbar[warp][par]);
                    if (lane == 0) mbar_arrive_expect(mb, halo_bytes);
                    const uint32_t ph = (uint32_t)((k - 1) >> 1) & 1u;
                    bool ok = mbar_test_wait(mb, ph);
                    if (!ok) {
                        const uint64_t t0 = global_ns();
                        while (!(ok = mbar_test_wait(mb, ph)) && global_ns() - t0 < kHaloWaitNs) {
                        }
                    }
                    if (!__all_sync(0xffffffffu, ok)) {
                        bad = true;
                        if (lane == 0) atomicAdd(&g_tiled_wait_failures, 1ull);
                    }
                }
                const int wl = lane * CPT;
                if (wl < H || wl >= H + O) {
                    const int side = wl < H ? 0 : 1;
                    const int off = wl < H ? wl : wl - H - O;
#pragma unroll
                    for (int c = 0; c < CPT; ++c) {
                        d2[c] = in[c] ? halo[warp][par][side][0][off + c] : T(0);
                        d1[c] = in[c] ? halo[warp][par][side][1][off + c] : T(0);
                    }
                }
            } else {
                // The owners of rows i0-1 and i0-2 stored them before arriving.
                cluster_sync_all();
                if (!own) {
                    const T* r1 = x + (int64_t)(i0 - 1) * nx + j0;
                    const T* r2 = r1 - nx;
#pragma unroll
                    for (int c = 0; c < CPT; ++c) {
                        d1[c] = in[c] ? __ldcg(r1 + c) : T(0);
                        d2[c] = in[c] ? __ldcg(r2 + c) : T(0);
                    }
                }
            }
        }
        if (i0 + H + PF <= nt) {  // no row or prefetch past the end
            int h = 0;
            if (i0 == 0) {
#pragma unroll
                for (int s = 0; s < PF; ++s) row(std::true_type{}, std::false_type{}, s, s);
                h = PF;
            }
            for (; h < H; h += PF) {
#pragma unroll
                for (int s = 0; s < PF; ++s)
                    row(std::false_type{}, std::false_type{}, i0 + h + s, s);
            }
        } else {
            for (int h = 0; h < H; h += PF) {
#pragma unroll
                for (int s = 0; s < PF; ++s) {
                    const int i = i0 + h + s;
                    if (i >= nt) break;  // uniform over the grid
                    if (i < 2) {
                        row(std::true_type{}, std::true_type{}, i, s);
                    } else {
                        row(std::false_type{}, std::true_type{}, i, s);
                    }
                }
            }
        }
        if constexpr (DSMEM) {
            // Rows i0+H-2 (d2) and i0+H-1 (d1) for the neighbours' next batch.
            if (push_addr != 0 && i0 + H < nt) {
                const uint32_t par = (uint32_t)((i0 / H + 1) & 1);
                const uint32_t a = push_addr + par * kHaloPar;
                const uint32_t m = push_mbar + par * 8u;
                push_cols<T, CPT>(a, m, d2);
                push_cols<T, CPT>(a + H * sizeof(T), m, d1);
            }
        }
    }
    if constexpr (DSMEM) cluster_sync_all();  // no CTA leaves while pushes may target it
}

template <typename T>
int tiled_launch(const void* kern, int clusters, int warps, const WaveDev<T>& g, const T* b,
                 T* x, uint32_t extra_wait, cudaStream_t st) {
    static thread_local const void* checked[64];
    static thread_local int nchecked = 0;
    bool seen = false;
    for (int q = 0; q < nchecked; ++q) seen |= checked[q] == kern;
    if (!seen) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (nchecked < 64) checked[nchecked++] = kern;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)clusters);
    cfg.blockDim = dim3((unsigned)(32 * warps));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)clusters;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // The cluster must fit on the device at once (its CTAs run together);
    // asked once per kernel and launch shape, so that launches made later
    // under stream capture query nothing.
    struct Fit {
        const void* kern;
        int clusters, warps, ok;
    };
    static thread_local Fit fits[64];
    static thread_local int nfits = 0;
    int ok = -1;
    for (int q = 0; q < nfits; ++q)
        if (fits[q].kern == kern && fits[q].clusters == clusters && fits[q].warps == warps)
            ok = fits[q].ok;
    if (ok < 0) {
        int n = 0;
        ok = cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n >= 1;
        cudaGetLastError();
        if (nfits < 64) fits[nfits++] = {kern, clusters, warps, ok};
    }
    if (!ok) return ODIL_ERR_SHAPE;
    void* args[] = {const_cast<WaveDev<T>*>(&g), &b, &x, &extra_wait};
    cfg.numAttrs = 2;  // the occupancy query above saw the cluster only
    if (cudaLaunchKernelExC(&cfg, kern, args) != cudaSuccess) {
        cudaGetLastError();
        return ODIL_ERR_LAUNCH;
    }
    return launch_status();
}

template <typename T, int CPT, int H, int PF, bool DSMEM>
int tiled_shape_fit(const WaveDev<T>& g, const T* b, T* x, int warps, uint32_t extra_wait,
                    bool table, cudaStream_t st) {
    constexpr int O = 32 * CPT - 2 * H;
    const int64_t tiles = (g.nx + O - 1) / O;
    if (warps < 1 || warps > kTiledMaxWarps) return ODIL_ERR_SHAPE;
    if (warps > tiles) warps = (int)tiles;
    const int64_t clusters = (tiles + warps - 1) / warps;
    if (clusters > 16) return ODIL_ERR_SHAPE;
    constexpr int vb = CPT * (int)sizeof(T) < 16 ? CPT * (int)sizeof(T) : 16;
    const bool vec = g.nx % CPT == 0 &&
                     ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(x)) % vb) == 0;
    const void* kern =
        vec ? reinterpret_cast<const void*>(wave_march_tiled_kernel<T, CPT, H, PF, true, DSMEM>)
            : reinterpret_cast<const void*>(wave_march_tiled_kernel<T, CPT, H, PF, false, DSMEM>);
    if (table) {  // FP32 only (the mixed solve from zero)
        if constexpr (sizeof(T) == 4) {
            kern = vec ? reinterpret_cast<const void*>(
                             wave_march_tiled_kernel<T, CPT, H, PF, true, DSMEM, true>)
                       : reinterpret_cast<const void*>(
                             wave_march_tiled_kernel<T, CPT, H, PF, false, DSMEM, true>);
        } else {
            return ODIL_ERR_ARG;
        }
    }
    return tiled_launch<T>(kern, (int)clusters, warps, g, b, x, extra_wait, st);
}

template <typename T, int CPT, int H, int PF, bool DSMEM>
int tiled_shape(const WaveDev<T>& g, const T* b, T* x, int warps, uint32_t extra_wait,
                bool table, cudaStream_t st) {
    // A ring above 512 bytes per thread spills (FP64 with cpt pf > 64).
    if constexpr (CPT * PF * sizeof(T) > 512) {
        return ODIL_ERR_SHAPE;
    } else {
        return tiled_shape_fit<T, CPT, H, PF, DSMEM>(g, b, x, warps, extra_wait, table, st);
    }
}

// Shapes as exchange * 1000000 + cpt * 10000 + halo * 100 + pf (exchange 0:
// cluster barrier and reload from global memory; 1: st.async into the
// neighbours' shared memory, needs 32 cpt - 2 halo >= halo).
template <typename T>
int tiled_dispatch(const odil_wave_params* p, const T* b, T* x, int cpt, int halo, int pf,
                   int warps, int exchange, uint32_t extra_wait, void* stream,
                   bool table = false) {
    WaveDev<T> g;
    int st = make_dev<T>(p, &g, false);
    if (st) return st;
    if (!b || !x) return ODIL_ERR_ARG;
    if (g.nx < 2) return ODIL_ERR_SHAPE;
    // Table mode: a lane holds at most one of columns 0 and nx - 1.
    if (table && g.nx <= cpt) return ODIL_ERR_SHAPE;
    if (cpt < 1 || cpt > 9 || halo < 1 || halo > 99 || pf < 1 || pf > 99 || exchange < 0 ||
        exchange > 1)
        return ODIL_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    const uint32_t e = extra_wait;
    switch (exchange * 1000000 + cpt * 10000 + halo * 100 + pf) {
        case 43216: return tiled_shape<T, 4, 32, 16, false>(g, b, x, warps, e, table, s);
        case 44816: return tiled_shape<T, 4, 48, 16, false>(g, b, x, warps, e, table, s);
        case 89616: return tiled_shape<T, 8, 96, 16, false>(g, b, x, warps, e, table, s);
        case 1021616: return tiled_shape<T, 2, 16, 16, true>(g, b, x, warps, e, table, s);
        case 1040808: return tiled_shape<T, 4, 8, 8, true>(g, b, x, warps, e, table, s);
        case 1041616: return tiled_shape<T, 4, 16, 16, true>(g, b, x, warps, e, table, s);
        case 1042408: return tiled_shape<T, 4, 24, 8, true>(g, b, x, warps, e, table, s);
        case 1043216: return tiled_shape<T, 4, 32, 16, true>(g, b, x, warps, e, table, s);
        case 1083216: return tiled_shape<T, 8, 32, 16, true>(g, b, x, warps, e, table, s);
        case 1086416: return tiled_shape<T, 8, 64, 16, true>(g, b, x, warps, e, table, s);
        default: return ODIL_ERR_SHAPE;
    }
}

}  // namespace
}  // namespace odil

using odil::tiled_dispatch;

ODIL_API int odil_wave_march_tiled_f32(const odil_wave_params* p, const float* b, float* x,
                                       int32_t cpt, int32_t halo, int32_t pf, int32_t warps,
                                       int32_t exchange, void* stream) {
    return tiled_dispatch<float>(p, b, x, cpt, halo, pf, warps, exchange, 0u, stream);
}

ODIL_API int odil_wave_march_tiled_table_f32(const odil_wave_params* p, const float* tbl,
                                             float* x, int32_t cpt, int32_t halo, int32_t pf,
                                             int32_t warps, int32_t exchange, void* stream) {
    return tiled_dispatch<float>(p, tbl, x, cpt, halo, pf, warps, exchange, 0u, stream, true);
}

ODIL_API int odil_wave_march_tiled_f64(const odil_wave_params* p, const double* b, double* x,
                                       int32_t cpt, int32_t halo, int32_t pf, int32_t warps,
                                       int32_t exchange, void* stream) {
    return tiled_dispatch<double>(p, b, x, cpt, halo, pf, warps, exchange, 0u, stream);
}

ODIL_API int odil_wave_march_tiled_planted_wait_f32(const odil_wave_params* p, const float* b,
                                                    float* x, int32_t cpt, int32_t halo,
                                                    int32_t pf, int32_t warps,
                                                    int32_t missing_bytes, void* stream) {
    if (missing_bytes <= 0 || missing_bytes > (1 << 16)) return ODIL_ERR_ARG;
    return tiled_dispatch<float>(p, b, x, cpt, halo, pf, warps, 1, (uint32_t)missing_bytes,
                                 stream);
}

ODIL_API int odil_wave_march_tiled_wait_failures(int64_t* count, int32_t reset) {
    if (!count) return ODIL_ERR_ARG;
    unsigned long long v = 0;
    if (cudaMemcpyFromSymbol(&v, odil::g_tiled_wait_failures, sizeof(v)) != cudaSuccess)
        return odil::launch_status();
    *count = (int64_t)v;
    if (reset) {
        v = 0;
        if (cudaMemcpyToSymbol(odil::g_tiled_wait_failures, &v, sizeof(v)) != cudaSuccess)
            return odil::launch_status();
    }
    return ODIL_OK;
}
