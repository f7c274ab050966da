// Many independent wave instances of uneven sizes solved together (the
// reference farms such runs out as separate processes, vary_wave.py:7-43).
// Fields of all instances are packed back to back (each instance starts on a
// 16-byte boundary); a device array of descriptors gives each instance's
// grid, wave speed, offsets and derived constants.
//
// One mixed-precision Newton epoch for the whole batch is two launches:
//   * batch_update_residual: FP64 u_out = u + d and rhs = float(-F(u_out))
//     over every cell of every instance (all SMs; the instance of a cell by
//     binary search over the start offsets);
//   * batch_march: a persistent FP32 forward-substitution kernel; each block
//     takes the next instance from an atomic work queue (instances ordered
//     largest first) and marches it with the single-instance device code.
// Both are stream-ordered, allocation-free and capture into a CUDA graph.
#include "wave_dev.cuh"

namespace odil {
namespace {
using namespace wavedev;

// Derived constants of every instance (double and float copies).
__global__ void batch_setup_kernel(odil_wave_instance* inst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    odil_wave_instance& d = inst[i];
    const double inv_dt = 1.0 / d.dt;
    const double inv_dx2 = 1.0 / (d.dx * d.dx);
    d.inv_dt = inv_dt;
    d.inv_dx2 = inv_dx2;
    d.c2 = d.c * d.c;
    d.dt2 = d.dt * d.dt;
    d.lam2 = d.c * d.c * d.dt * d.dt * inv_dx2;
    d.a = inv_dt * inv_dt;
    d.b = d.c2 * inv_dx2;
    d.half_dt = 0.5 * d.dt;
    const PairCoef k = pair_coef_dev(d.a, d.b);
    d.ah = k.ah;
    d.al = k.al;
    d.ch = k.ch;
    d.cl = k.cl;
    d.bh = k.bh;
    d.bl = k.bl;
}

template <typename T>
__device__ __forceinline__ WaveDev<T> dev_of(const odil_wave_instance& d, const T* init_u,
                                             const T* init_ut, const T* left_u,
                                             const T* right_u) {
    WaveDev<T> g;
    g.nt = (int)d.nt;
    g.nx = (int)d.nx;
    // Copies of constants computed once by batch_setup_kernel (no FP64
    // arithmetic per block or row).
    g.inv_dt = (T)d.inv_dt;
    g.inv_dx2 = (T)d.inv_dx2;
    g.c2 = (T)d.c2;
    g.half_dt = (T)d.half_dt;
    g.A = (T)d.a;
    g.B = (T)d.b;
    g.dt2 = (T)d.dt2;
    g.lam2 = (T)d.lam2;
    g.init_u = init_u ? init_u + d.offset_x : nullptr;
    g.init_ut = init_ut ? init_ut + d.offset_x : nullptr;
    g.left_u = left_u ? left_u + d.offset_t : nullptr;
    g.right_u = right_u ? right_u + d.offset_t : nullptr;
    return g;
}

// Instance holding packed cell k (starts sorted ascending), or -1 in padding.
__device__ __forceinline__ int find_inst(const odil_wave_instance* __restrict__ inst, int n,
                                         int64_t k) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&inst[mid].offset) <= k) lo = mid; else hi = mid - 1;
    }
    const int64_t off = __ldg(&inst[lo].offset);
    const int64_t cells = __ldg(&inst[lo].nt) * __ldg(&inst[lo].nx);
    return (k >= off && k < off + cells) ? lo : -1;
}

__global__ void __launch_bounds__(256) batch_update_residual_kernel(
    odil_wave_batch b, const double* __restrict__ u, const float* __restrict__ d,
    double* __restrict__ uout, float* __restrict__ rhs) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const double* iu = (const double*)b.init_u;
    const double* iut = (const double*)b.init_ut;
    const double* lu = (const double*)b.left_u;
    const double* ru = (const double*)b.right_u;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < b.total_cells;
         k += stride) {
        const int q = find_inst(b.inst, b.ninst, k);
        if (q < 0) {
            rhs[k] = 0.f;
            if (d) uout[k] = 0.0;
            continue;
        }
        const odil_wave_instance desc = b.inst[q];
        const WaveDev<double> g = dev_of<double>(desc, iu, iut, lu, ru);
        const int64_t local = k - desc.offset;
        const int i = (int)(local / g.nx);
        const int j = (int)(local - (int64_t)i * g.nx);
        const double* ub = u + desc.offset;
        const float* db = d ? d + desc.offset : nullptr;
        auto val = [&](int ii, int jj) -> double {
            const int64_t kk = (int64_t)ii * g.nx + jj;
            double v = __ldg(ub + kk);
            if (db) v += (double)__ldg(db + kk);
            return v;
        };
        const double uc = val(i, j);
        double utm = 0, utmm = 0, uxm = 0, uxp = 0;
        if (i >= 1) {
            utm = val(i - 1, j);
            uxm = val(i - 1, j == 0 ? g.nx - 1 : j - 1);
            uxp = val(i - 1, j + 1 == g.nx ? 0 : j + 1);
        }
        if (i >= 2) utmm = val(i - 2, j);
        const double f = wave_f(g, i, j, uc, utm, utmm, uxm, uxp);
        if (d) uout[k] = uc;
        rhs[k] = (float)(-f);
    }
}


// Interior cells of all instances, one warp per packed time row (the row's
// instance from the row table), lanes over the columns 1 .. nx-2 of rows
// >= 2.  KIND 0: rhs = 0 there (F(0) vanishes inside); KIND 1: rhs =
// float(-F(hi + lo)) in the float-pair form (wave_dev.cuh).  No FP64.
template <int KIND>
__global__ void __launch_bounds__(256) batch_rows_kernel(odil_wave_batch b,
                                                         const float* __restrict__ hi,
                                                         const float* __restrict__ lo,
                                                         float* __restrict__ rhs) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= b.total_rows) return;
    const odil_wave_instance& d = b.inst[__ldg(b.row_inst + r)];
    const int i = (int)(r - d.offset_t);
    const int nx = (int)d.nx;
    if (i < 2) return;
    const int64_t off = d.offset;
    float* rrow = rhs + off + (int64_t)i * nx;
    if (KIND == 0) {
        for (int j = 1 + lane; j < nx - 1; j += 32) rrow[j] = 0.f;
    } else {
        PairCoef k;
        k.ah = d.ah;
        k.al = d.al;
        k.ch = d.ch;
        k.cl = d.cl;
        k.bh = d.bh;
        k.bl = d.bl;
        const float* h = hi + off;
        const float* l = lo ? lo + off : nullptr;
        for (int j = 1 + lane; j < nx - 1; j += 32)
            rrow[j] = pair_interior_rhs(k, h, l, (int64_t)i * nx + j, nx);
    }
}

// Boundary cells of all instances, one thread per cell (full warps): the
// instance by binary search over the boundary offsets, the cell by
// bnd_cell, the value in FP64.
template <int KIND>
__global__ void __launch_bounds__(256) batch_bnd_kernel(odil_wave_batch b,
                                                        const float* __restrict__ hi,
                                                        const float* __restrict__ lo,
                                                        float* __restrict__ rhs) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.total_bnd) return;
    int a = 0, z = b.ninst - 1;
    while (a < z) {
        const int mid = (a + z + 1) >> 1;
        if (__ldg(b.bnd_off + mid) <= t) a = mid; else z = mid - 1;
    }
    const odil_wave_instance desc = b.inst[a];
    const WaveDev<double> g =
        dev_of<double>(desc, (const double*)b.init_u, (const double*)b.init_ut,
                       (const double*)b.left_u, (const double*)b.right_u);
    int i, j;
    bnd_cell(t - __ldg(b.bnd_off + a), g.nt, g.nx, &i, &j);
    PairCoef k;
    k.ah = desc.ah;
    k.al = desc.al;
    k.ch = desc.ch;
    k.cl = desc.cl;
    k.bh = desc.bh;
    k.bl = desc.bl;
    const int64_t off = desc.offset;
    rhs[off + (int64_t)i * g.nx + j] =
        bnd_cell_rhs<KIND>(g, k, hi ? hi + off : nullptr, lo ? lo + off : nullptr, i, j);
}

template <int KIND>
int launch_rhs(const odil_wave_batch* b, const float* hi, const float* lo, float* rhs,
               cudaStream_t s) {
    if (!b->row_inst || b->total_rows < 1 || !b->bnd_off || b->total_bnd < 1)
        return ODIL_ERR_ARG;
    batch_rows_kernel<KIND><<<(unsigned)((b->total_rows + 7) / 8), 256, 0, s>>>(*b, hi, lo, rhs);
    batch_bnd_kernel<KIND><<<(unsigned)((b->total_bnd + 255) / 256), 256, 0, s>>>(*b, hi, lo,
                                                                                rhs);
    return launch_status();
}

template <int CPT, int PF>
__global__ void __launch_bounds__(1024) batch_march_kernel(odil_wave_batch b,
                                                           const float* __restrict__ rhs,
                                                           float* __restrict__ x,
                                                           unsigned* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sh_q;
    for (;;) {
        if (threadIdx.x == 0) sh_q = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int q = sh_q;
        __syncthreads();
        if (q >= b.ninst) break;
        const int idx = __ldg(b.order + q);
        const odil_wave_instance desc = b.inst[idx];
        const WaveDev<float> g = dev_of<float>(desc, nullptr, nullptr, nullptr, nullptr);
        const float* bb = rhs + desc.offset;
        float* xx = x + desc.offset;
        if (g.nx % CPT == 0) {
            march_instance<float, CPT, PF, true>(g, bb, xx, smem_raw);
        } else {
            march_instance<float, CPT, PF, false>(g, bb, xx, smem_raw);
        }
        __syncthreads();
    }
}

// The whole mixed Newton of the batch in one persistent launch.  Each block
// takes the next instance (largest first) from the work queue and runs its
// epochs as marches whose right-hand sides are formed inside the march, row
// by row, from the previous iterate:
//   march 1 (SRC 0): rhs = float(-F(0)), zero inside;
//   march 2 (SRC 1): rhs = float(-F(hi)) inside, in float pairs;
//   march e > 2 (SRC 2): rhs = float(-F(hi + lo)) inside, and lo += x;
// the boundary cells' values (rows 0, 1, columns 0 and nx-1) in FP64,
// computed by the whole block into a table before each march (the table
// lives in the instance's rhs region).  The iterate's rows stream into
// shared-memory rings by cp.async, PF - 2 rows ahead of the march step,
// so rows i + 1, i and i - 1 are resident when the right-hand side of row
// i + 1 is formed during step i; the column-table entries ride in
// the same copy groups.  The last march writes u = hi + lo in FP64 as it
// goes (one FP64 add of the two widened floats: exact wherever the sum fits
// a double, and the value pair_to_f64 forms with integer instructions; the
// FP64 pipe is otherwise idle here, the integer form would load the issue
// slots the march needs), so its correction never reaches memory:
// with two epochs an instance costs a 4-byte write and read of hi and the
// 8-byte write of u per cell.  The arithmetic is that of the multi-launch
// path (batch_rows / batch_bnd, batch_march, pair_to_f64), so the results
// are bitwise the same.  Values written in this kernel are read back
// through L2 (ld.global.cg) or by the block that wrote them after a block
// barrier; instances start on 128-byte boundaries (the host's packing), so
// no L1 line holds two instances' data.  Counters: [0] the work queue,
// [1] blocks done; the last block to finish resets both, so the workspace
// needs zeroing once, before the first launch.

struct FusedSmem {
    float* ringh;  // [max_nx][PF + 1] rows of hi
    float* ringl;  // [max_nx][PF + 1] rows of lo (SRC 2)
    float* tring;  // [2][PF] column-table entries (column 0, column nx-1)
    float* edge;   // [2 parity][2 end][kMarchMaxWarps]
};

// One march of the fused solve (see above).  x: the float result (hi for
// SRC 0, lo otherwise; lo is updated in place for SRC 2) unless LAST, when
// u = hi + lo goes to uo in FP64 instead.  The row step is that of
// march_instance; the right-hand side of row i + 1 is formed during step i
// and the FP64 value of row i - 1 is written during step i, both off the
// row-to-row dependency chain (independent of the step's march arithmetic,
// so their latency hides behind it).  Only the warps that hold columns of
// this instance march (blocks are sized for the widest instance of the
// batch); they meet at named barrier 1, the others wait at the block
// barrier at the end.  Ring layout [column][PF + 1]: a slot is an immediate
// offset, and a warp's 32 columns fall in distinct banks.
template <int SRC, bool LAST, int CPT, int PF, bool VEC>
__device__ __forceinline__ void fused_march(const WaveDev<float>& g, const PairCoef& k,
                                            const float* tbl, const float* hs,
                                            const float* ls, float* x, double* uo,
                                            const FusedSmem& sm) {
    static_assert(PF % 2 == 0 && PF >= 4, "row parity follows the ring slot");
    constexpr int RS = PF + 1;  // ring stride per column
    const int nx = g.nx, nt = g.nt;
    const int nact = ((nx + CPT - 1) / CPT + 31) & ~31;  // marching threads
    if ((int)threadIdx.x < nact) {
        const int lane = threadIdx.x & 31;
        const int warp = threadIdx.x >> 5;
        const int nwarp = nact >> 5;
        const int j0 = threadIdx.x * CPT;
        float kxm[CPT], ktm[CPT], kxp[CPT], d1[CPT], d2[CPT];
        // Own columns of the iterate: hb / lb row i, hc / lc row i - 1 (at
        // the start of step i); rc: right-hand side of row i; pend: result
        // of row i - 1 (its FP64 write is pending).
        float hb[CPT], hc[CPT], lb[CPT], lc[CPT], rc[CPT], pend[CPT], r1[CPT];
        const float* hcol[CPT];  // ring columns (own, clamped into the row)
        const float* lcol[CPT];
        bool in[CPT];       // column inside the row
        unsigned bcol = 0;  // bit c: column j0 + c is 0 or nx - 1
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const int j = j0 + c;
            in[c] = j < nx;
            const int jj = in[c] ? j : 0;
            // Columns past the row end march zeros: no coupling, zero rhs.
            ktm[c] = in[c] ? k_tm<float>(jj, nx) : 0.f;
            kxm[c] = in[c] ? k_xm<float>(jj, nx) : 0.f;
            kxp[c] = in[c] ? k_xp<float>(jj, nx) : 0.f;
            d1[c] = 0.f;
            d2[c] = 0.f;
            hb[c] = hc[c] = lb[c] = lc[c] = pend[c] = 0.f;
            const int jc = in[c] ? j : nx - 1;
            hcol[c] = sm.ringh + jc * RS;
            lcol[c] = sm.ringl + jc * RS;
            if (j == 0 || j == nx - 1) bcol |= 1u << c;
            rc[c] = in[c] ? __ldcg(tbl + j) : 0.f;  // row 0: all boundary
            r1[c] = (in[c] && nt >= 2) ? __ldcg(tbl + nx + j) : 0.f;
        }
        const int jl = j0 > 0 ? (j0 - 1 < nx - 1 ? j0 - 1 : nx - 1) : 0;
        const int jr = j0 + CPT < nx ? j0 + CPT : nx - 1;
        const float* hl = sm.ringh + jl * RS;
        const float* hr = sm.ringh + jr * RS;
        const float* ll = sm.ringl + jl * RS;
        const float* lr = sm.ringl + jr * RS;
        const bool own_l = j0 == 0;
        const bool own_r = in[0] && nx - 1 < j0 + CPT;
        const int wl = warp > 0 ? warp - 1 : 0;
        const int wr = warp + 1 < nwarp ? warp + 1 : warp;
        const bool use_l = lane == 0, use_r = lane == 31;
        const bool self_r = nx == 1;
        float* edge = sm.edge;
        for (int e = threadIdx.x; e < 4 * kMarchMaxWarps; e += nact) edge[e] = 0.f;
        // Copy sources of the next row to issue.  The table follows the
        // bnd_cell sequence: rows 0 and 1, then the cc (= min(nx, 2))
        // column entries (column 0, then nx - 1) of each row from 2 on.
        const float* hsrc = hs + j0;
        const float* lsrc = ls + j0;
        const int cc = nx < 2 ? nx : 2;
        const float* tsrc = tbl + (nt < 2 ? nt : 2) * nx;  // column entries of row 2
        float* dst = x + j0;
        double* udst = uo + j0;
        auto bar = [&]() { asm volatile("bar.sync 1, %0;" ::"r"(nact) : "memory"); };
        // Copy group of row rr into ring slot `slot` (one group per row,
        // empty past the last row).
        auto issue = [&](int rr, int slot) {
            if (rr < nt) {
#pragma unroll
                for (int c = 0; c < CPT; ++c) {
                    if (in[c]) {
                        if constexpr (SRC >= 1)
                            cp_async_n(sm.ringh + (j0 + c) * RS + slot, hsrc + c, 4);
                        if constexpr (SRC == 2)
                            cp_async_n(sm.ringl + (j0 + c) * RS + slot, lsrc + c, 4);
                    }
                }
                if (rr >= 2) {
                    if (own_l) cp_async_n(sm.tring + slot, tsrc, 4);
                    if (own_r) cp_async_n(sm.tring + PF + slot, tsrc + (cc - 1), 4);
                    tsrc += cc;
                }
            }
            hsrc += nx;
            lsrc += nx;
            cp_async_commit();
        };
        // FP64 write of a row (result out, iterate h / l of the row): the
        // widening is exact and the FP64 add rounds only where the sum does
        // not fit a double, as pair_sum_exact does.
        auto write_u = [&](double* to, const float* out, const float* h, const float* l) {
            double uv[CPT];
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                if constexpr (SRC == 0) {
                    uv[c] = (double)out[c];
                } else if constexpr (SRC == 1) {
                    uv[c] = __dadd_rn((double)h[c], (double)out[c]);
                } else {
                    uv[c] = __dadd_rn((double)h[c], (double)__fadd_rn(l[c], out[c]));
                }
            }
            if constexpr (VEC && CPT % 2 == 0) {
                if (in[0]) {
#pragma unroll
                    for (int c = 0; c < CPT; c += 2)
                        *reinterpret_cast<double2*>(to + c) = make_double2(uv[c], uv[c + 1]);
                }
            } else {
#pragma unroll
                for (int c = 0; c < CPT; ++c)
                    if (in[c]) to[c] = uv[c];
            }
        };
        // Rows 0 .. PF - 3 in flight; row 0 landed (own columns) before the
        // first step, so step i finds row i resident and waits for row i + 1.
#pragma unroll
        for (int s = 0; s < PF - 2; ++s) issue(s, s);
        cp_async_wait<PF - 3>();
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            if constexpr (SRC >= 1) hb[c] = hcol[c][0];
            if constexpr (SRC == 2) lb[c] = lcol[c][0];
        }
        bar();
        auto row = [&](auto gen_tag, int i, int s) {
            constexpr bool GEN = decltype(gen_tag)::value;
            const int sn = (s + 1) % PF;  // slot of row i + 1
            issue(i + PF - 2, (s + PF - 2) % PF);
            const float c_rhs = GEN ? (i == 0 ? 1.f : g.dt2) : g.dt2;
            const float c_d1 = GEN ? (i == 1 ? 1.f : 2.f) : 2.f;
            const float c_lam = GEN ? (i == 0 ? 0.f : g.lam2) : g.lam2;
            const float* eprv = edge + ((s & 1) ^ 1) * 2 * kMarchMaxWarps;
            const float el = eprv[kMarchMaxWarps + wl];
            const float er = eprv[wr];
            const float sl = __shfl_up_sync(0xffffffffu, d1[CPT - 1], 1);
            const float sr = __shfl_down_sync(0xffffffffu, d1[0], 1);
            const float left = use_l ? el : sl;
            const float right = self_r ? d1[0] : (use_r ? er : sr);
            float out[CPT];
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                const float xm = c == 0 ? left : d1[c - 1];
                const float xp = c == CPT - 1 ? right : d1[c + 1];
                const float tprev = c_d1 * d1[c] - d2[c];
                out[c] = c_rhs * rc[c] + tprev +
                         c_lam * (kxm[c] * xm - ktm[c] * d1[c] + kxp[c] * xp);
            }
            if constexpr (!LAST) {
                float res[CPT];
#pragma unroll
                for (int c = 0; c < CPT; ++c)
                    res[c] = SRC == 2 ? __fadd_rn(lb[c], out[c]) : out[c];
                if constexpr (VEC) {
                    if (in[0]) {
                        Chunk<float, CPT> ch;
#pragma unroll
                        for (int c = 0; c < CPT; ++c) ch.v[c] = res[c];
                        *reinterpret_cast<Chunk<float, CPT>*>(dst) = ch;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < CPT; ++c)
                        if (in[c]) dst[c] = res[c];
                }
            }
            float* ecur = edge + (s & 1) * 2 * kMarchMaxWarps;
            if (use_l) ecur[warp] = out[0];
            if (use_r) ecur[kMarchMaxWarps + warp] = out[CPT - 1];
            // Row i - 1's FP64 write.
            if constexpr (LAST) {
                if (!GEN || i >= 1) write_u(udst - nx, pend, hc, lc);
            }
            // Right-hand side of row i + 1 from rows i + 1, i, i - 1 (row
            // i + 1 of this thread landed here; rows i and i - 1 of every
            // thread are resident since the last barriers).
            cp_async_wait<PF - 3>();
            float ha[CPT], la[CPT], rn[CPT];
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                ha[c] = SRC >= 1 ? hcol[c][sn] : 0.f;
                la[c] = SRC == 2 ? lcol[c][sn] : 0.f;
            }
            float hm = 0.f, hp = 0.f, lm = 0.f, lp = 0.f;  // row i at j0 - 1, j0 + CPT
            if constexpr (SRC >= 1) {
                hm = hl[s];
                hp = hr[s];
            }
            if constexpr (SRC == 2) {
                lm = ll[s];
                lp = lr[s];
            }
            (void)hm, (void)hp, (void)lm, (void)lp;
            const float tl = sm.tring[sn], tr = sm.tring[PF + sn];
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                float v = 0.f;
                if constexpr (SRC >= 1) {
                    const float vm = c == 0 ? hm : hb[c - 1];
                    const float vp = c == CPT - 1 ? hp : hb[c + 1];
                    const float wm = c == 0 ? lm : lb[c - 1];
                    const float wp = c == CPT - 1 ? lp : lb[c + 1];
                    v = pair_rhs_vals(k, ha[c], hc[c], hb[c], vm, vp, la[c], lc[c], lb[c], wm, wp);
                }
                if ((bcol >> c) & 1u) v = j0 + c == 0 ? tl : tr;
                if (GEN && i + 1 == 1) v = r1[c];
                rn[c] = in[c] ? v : 0.f;
            }
            dst += nx;
            udst += nx;
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                d2[c] = d1[c];
                d1[c] = out[c];
                pend[c] = out[c];
                hc[c] = hb[c];
                hb[c] = ha[c];
                lc[c] = lb[c];
                lb[c] = la[c];
                rc[c] = rn[c];
            }
            bar();
        };
        for (int i0 = 0; i0 < nt; i0 += PF) {
            if (i0 == 0 || i0 + PF > nt) {
#pragma unroll
                for (int s = 0; s < PF; ++s) {
                    if (i0 + s >= nt) break;
                    row(std::true_type{}, i0 + s, s);
                }
            } else {
#pragma unroll
                for (int s = 0; s < PF; ++s) row(std::false_type{}, i0 + s, s);
            }
        }
        // The last row's FP64 write (hc / lc hold its iterate after the
        // shift).
        if constexpr (LAST) write_u(udst - nx, pend, hc, lc);
        cp_async_wait<0>();
    }
    __syncthreads();
}

// Threads per block of the fused solve: the pair stencil, three rows of the
// iterate and the march state need more than the 64 registers a 1024-thread
// block leaves once a thread owns more than one column.
template <int CPT>
constexpr int batch_solve_max_threads() { return CPT == 1 ? 1024 : 512; }

template <int CPT, int PF>
__global__ void __launch_bounds__(batch_solve_max_threads<CPT>()) batch_solve_kernel(
    odil_wave_batch b, int epochs, float* __restrict__ rhs, float* __restrict__ hi, float* lo,
    double* __restrict__ u, unsigned* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sh_q;
    const int nthr = blockDim.x;
    FusedSmem sm;
    const int ring = b.max_nx * (PF + 1);
    sm.ringh = reinterpret_cast<float*>(smem_raw);
    sm.ringl = sm.ringh + ring;
    sm.tring = sm.ringl + (epochs > 2 ? ring : 0);
    sm.edge = sm.tring + 2 * PF;
    const double* iu = (const double*)b.init_u;
    const double* iut = (const double*)b.init_ut;
    const double* lu = (const double*)b.left_u;
    const double* ru = (const double*)b.right_u;
    for (;;) {
        if (threadIdx.x == 0) sh_q = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int q = sh_q;
        __syncthreads();
        if (q >= b.ninst) break;
        const int idx = __ldg(b.order + q);
        const odil_wave_instance desc = b.inst[idx];
        const WaveDev<double> g64 = dev_of<double>(desc, iu, iut, lu, ru);
        const WaveDev<float> g32 = dev_of<float>(desc, nullptr, nullptr, nullptr, nullptr);
        const int nt = g32.nt, nx = g32.nx;
        const int64_t off = desc.offset;
        PairCoef k;
        k.ah = desc.ah;
        k.al = desc.al;
        k.ch = desc.ch;
        k.cl = desc.cl;
        k.bh = desc.bh;
        k.bl = desc.bl;
        float* tb = rhs + off;
        float* h = hi + off;
        float* l = lo ? lo + off : nullptr;
        double* uo = u + off;
        const int64_t nb = bnd_count(nt, nx);
        // Boundary table of the current iterate (KIND 0: u = 0; 1: hi + lo).
        auto table = [&](auto kind_tag, const float* lp) {
            constexpr int KIND = decltype(kind_tag)::value;
            for (int64_t t = threadIdx.x; t < nb; t += nthr) {
                int i, j;
                bnd_cell(t, nt, nx, &i, &j);
                tb[t] = bnd_cell_rhs<KIND, false>(g64, k, h, lp, i, j);
            }
            __syncthreads();
        };
        // The first march (no stencil of an iterate) takes two columns per
        // thread where the others take one: half the per-row overhead.
        auto march = [&](auto src_tag, auto last_tag, float* x) {
            constexpr int SRC = decltype(src_tag)::value;
            constexpr bool LAST = decltype(last_tag)::value;
            constexpr int C = (SRC == 0 && CPT == 1) ? 2 : CPT;
            if (nx % C == 0) {
                fused_march<SRC, LAST, C, PF, true>(g32, k, tb, h, l, x, uo, sm);
            } else {
                fused_march<SRC, LAST, C, PF, false>(g32, k, tb, h, l, x, uo, sm);
            }
        };
        using I0 = std::integral_constant<int, 0>;
        using I1 = std::integral_constant<int, 1>;
        using I2 = std::integral_constant<int, 2>;
        table(I0{}, nullptr);
        if (epochs == 1) {
            march(I0{}, std::true_type{}, h);
        } else {
            march(I0{}, std::false_type{}, h);
            for (int e = 2; e <= epochs; ++e) {
                table(I1{}, e > 2 ? l : nullptr);
                if (e == 2) {
                    if (e == epochs) march(I1{}, std::true_type{}, l);
                    else march(I1{}, std::false_type{}, l);
                } else {
                    if (e == epochs) march(I2{}, std::true_type{}, l);
                    else march(I2{}, std::false_type{}, l);
                }
            }
        }
        // The padding up to the next instance is zero, as the multi-launch
        // path leaves it.
        const int64_t pad_end = idx + 1 < b.ninst ? b.inst[idx + 1].offset : b.total_cells;
        for (int64_t c = off + (int64_t)nt * nx + threadIdx.x; c < pad_end; c += nthr) u[c] = 0.0;
        __syncthreads();
    }
    // The last block out resets the queue for the next launch.
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(counter + 1, 1u) == gridDim.x - 1) {
            counter[0] = 0u;
            counter[1] = 0u;
            __threadfence();
        }
    }
}

// Shared memory of the fused solve: the hi ring (and the lo ring for more
// than two epochs), the column-table ring and the edge words.
template <int PF>
size_t batch_solve_smem(int max_nx, int epochs) {
    const size_t ring = (size_t)max_nx * (PF + 1) * 4;
    return ring * (epochs > 2 ? 2 : 1) + 2 * PF * 4 + 4 * kMarchMaxWarps * 4;
}

template <int CPT, int PF>
int launch_batch_solve(const odil_wave_batch* b, int epochs, float* rhs, float* hi, float* lo,
                       double* u, unsigned* counter, int threads, int blocks, cudaStream_t st) {
    if ((int64_t)threads * CPT < b->max_nx || threads > batch_solve_max_threads<CPT>())
        return ODIL_ERR_SHAPE;
    const size_t smem = batch_solve_smem<PF>(b->max_nx, epochs);
    if (smem > 200 * 1024) return ODIL_ERR_SHAPE;
    auto kern = batch_solve_kernel<CPT, PF>;
    ensure_dynamic_smem(reinterpret_cast<const void*>(kern), smem);
    kern<<<blocks, threads, smem, st>>>(*b, epochs, rhs, hi, lo, u, counter);
    return launch_status();
}

int check_batch(const odil_wave_batch* b) {
    if (!b) return ODIL_ERR_ARG;
    if (b->ninst < 1 || b->total_cells < 1 || b->max_nx < 1 || b->max_nx > 4096)
        return ODIL_ERR_SHAPE;
    if (!b->inst || !b->order) return ODIL_ERR_ARG;
    return ODIL_OK;
}

inline int sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 132;
}

template <int CPT, int PF>
int launch_batch_march(const odil_wave_batch* b, const float* rhs, float* x, unsigned* counter,
                       int threads, int blocks, cudaStream_t st) {
    if ((int64_t)threads * CPT < b->max_nx) return ODIL_ERR_SHAPE;
    const size_t smem = march_ring_smem_bytes<float>(b->max_nx, PF);
    if (smem > 200 * 1024) return ODIL_ERR_SHAPE;
    auto kern = batch_march_kernel<CPT, PF>;
    ensure_dynamic_smem(reinterpret_cast<const void*>(kern), smem);
    cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    kern<<<blocks, threads, smem, st>>>(*b, rhs, x, counter);
    return launch_status();
}

// Fused loss + adjoint gradient of every instance in one launch (FP32).
// Work items are strips of BLG_OUT output columns by BLG_TY rows, numbered
// instance by instance, row tile by row tile (tile_start: first item of
// each instance, tile_start[ninst] = total; tile_inst: the instance of each
// item); one warp per item, BLG_WARPS independent warps per block.
//
// Lane l holds BLG_V = 4 contiguous columns c0 - 1 + 4 l + j of a 128-column
// window (the first and last column are halo; lanes 0 and 31 also read one
// column beyond, for the halo's residual).  Rows of uneven widths give no
// 16-byte alignment, so rows stream into a per-warp ring of BLG_R shared-
// memory rows by 4-byte cp.async copies, BLG_R - 1 rows in flight per warp
// without holding registers; the ring row places the lane's four columns on
// a 16-byte boundary, so each lane reads them back with one 16-byte shared
// load.  Per row the warp forms the residual of the row (x-neighbours by two
// shuffles) and the gradient of the row two above from the residual rows
// below it (two more shuffles).  Column classes are per-lane constants (the
// d f/d u coefficients of the J^T gather, formed once per item), so every
// cell takes the same instructions; only the residual at columns 0 and
// nx - 1 (one lane each: the boundary extrapolation), rows 0, 1 of the
// residual and rows 0, nt - 2, nt - 1 of the gradient take the general
// per-cell functions.  96 registers (5 blocks of 4 warps per SM) hold it
// without spills: 20 warps x 7 rows in flight per SM.
constexpr int BLG_V = 4;
constexpr int BLG_OUT = 32 * BLG_V - 2;  // output columns per item
constexpr int BLG_TY = 32;
constexpr int BLG_WARPS = 4;
constexpr int BLG_R = 8;      // ring rows per warp (power of two)
// floats per ring row: [3] left extra column, [4 + 4 l + j] the lanes'
// columns, [132] right extra column, [133] / [134] the boundary values
// left_u / right_u of the row above (for the residual at columns 0, nx-1)
constexpr int BLG_ROW = 136;

// Residual of an interior cell (row >= 2, 0 < column < nx - 1): the
// expression of wave_f_with for such cells.
__device__ __forceinline__ float blg_f(const WaveDev<float>& g, float u, float utm, float utmm,
                                      float uxm, float uxp) {
    const float u_t_tm = (u - utm) * g.inv_dt;
    const float u_t_tmm = (utm - utmm) * g.inv_dt;
    const float u_tt = (u_t_tm - u_t_tmm) * g.inv_dt;
    const float u_xx = (uxm - 2.f * utm + uxp) * g.inv_dx2;
    return u_tt - g.c2 * u_xx;
}

__global__ void __launch_bounds__(BLG_WARPS * 32, 5) batch_loss_grad_kernel(
    const odil_wave_instance* __restrict__ inst, const int32_t* __restrict__ tile_inst,
    const int64_t* __restrict__ tile_start, int64_t nitems, const float* __restrict__ iu,
    const float* __restrict__ iut, const float* __restrict__ lu, const float* __restrict__ ru,
    const float* __restrict__ u, float* __restrict__ grad, double* __restrict__ partials) {
    constexpr int V = BLG_V;
    constexpr int NQ = BLG_TY + 4;  // rows a0 - 2 .. a0 + BLG_TY + 1
    __shared__ __align__(16) float ring_all[BLG_WARPS][BLG_R][BLG_ROW];
    const int lane = threadIdx.x & 31;
    const int64_t item = (int64_t)blockIdx.x * BLG_WARPS + (threadIdx.x >> 5);
    if (item >= nitems) return;  // the whole warp
    float* __restrict__ ring = &ring_all[threadIdx.x >> 5][0][0];
    const int qi = __ldg(tile_inst + item);
    const odil_wave_instance& d = inst[qi];
    WaveDev<float> g;
    g.nt = (int)d.nt;
    g.nx = (int)d.nx;
    g.inv_dt = (float)d.inv_dt;
    g.inv_dx2 = (float)d.inv_dx2;
    g.c2 = (float)d.c2;
    g.half_dt = (float)d.half_dt;
    g.A = (float)d.a;
    g.B = (float)d.b;
    g.dt2 = (float)d.dt2;
    g.lam2 = (float)d.lam2;
    g.init_u = iu + d.offset_x;
    g.init_ut = iut + d.offset_x;
    g.left_u = lu + d.offset_t;
    g.right_u = ru + d.offset_t;
    const int nt = g.nt, nx = g.nx;
    const float A = g.A, B = g.B;
    const int nsx = (nx + BLG_OUT - 1) / BLG_OUT;
    const int t = (int)(item - __ldg(tile_start + qi));
    const int ty = t / nsx, sx = t - ty * nsx;
    const int c0 = sx * BLG_OUT;       // first output column
    const int a0 = ty * BLG_TY;        // first output row
    const int cb = c0 - 1 + V * lane;  // column of this lane's element 0
    const float* __restrict__ ui = u + d.offset;
    float* __restrict__ gi = grad + d.offset;
    // Narrow grids (nx < 3) have no interior column: general functions only.
    const bool gen = nx < 3;
    // 2 / N in FP32 (N = nt nx < 2^24 is exact): no FP64 division per item.
    const float gscale = 2.f / ((float)nt * (float)nx);
    int off[V];
    float ctm[V], kxm1[V], kxp1[V];
    unsigned outm = 0, fixm = 0;
#pragma unroll
    for (int j = 0; j < V; ++j) {
        const int col = cb + j;
        const int cw = wrapn(col, nx);
        off[j] = cw;
        const int bp = (cw + 1 == nx) ? 0 : cw + 1;
        const int bm = (cw == 0) ? nx - 1 : cw - 1;
        ctm[j] = -2.f * A + B * k_tm<float>(cw, nx);
        kxm1[j] = k_xm<float>(bp, nx);
        kxp1[j] = k_xp<float>(bm, nx);
        if (col >= c0 && col < c0 + BLG_OUT && col < nx) outm |= 1u << j;
        if (col == 0 || col == nx - 1) fixm |= 1u << j;
    }
    // Lanes 0 and 31 also copy the column beyond the window's edge.
    const bool xl = lane == 0 || lane == 31;
    const int offe = lane == 0 ? wrapn(c0 - 2, nx) : wrapn(c0 + 32 * V - 1, nx);
    const int xe = lane == 0 ? 3 : 4 + 32 * V;  // its ring index
    // Lanes holding column 0 / nx - 1 also stream left_u / right_u.
    bool has_l = false, has_r = false;
#pragma unroll
    for (int j = 0; j < V; ++j) {
        has_l |= cb + j == 0;
        has_r |= cb + j == nx - 1;
    }
    // Row q (r = a0 - 2 + q) into ring slot q mod BLG_R; rows outside the
    // grid are zero.  Every call commits one group (empty past the tile), so
    // the wait below counts rows.
    auto issue = [&](int q) {
        if (q < NQ) {
            const int r = a0 - 2 + q;
            float* to = ring + (q & (BLG_R - 1)) * BLG_ROW;
            if (r >= 0 && r < nt) {
                const float* row = ui + (int64_t)r * nx;
#pragma unroll
                for (int j = 0; j < V; ++j) cp_async_n(to + 4 + V * lane + j, row + off[j], 4);
                if (xl) cp_async_n(to + xe, row + offe, 4);
                if (r >= 1 && has_l) cp_async_n(to + 133, g.left_u + (r - 1), 4);
                if (r >= 1 && has_r) cp_async_n(to + 134, g.right_u + (r - 1), 4);
            } else {
#pragma unroll
                for (int j = 0; j < V; ++j) to[4 + V * lane + j] = 0.f;
                if (xl) to[xe] = 0.f;
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int q = 0; q < BLG_R - 1; ++q) issue(q);

    float u1[V], u2[V], f1[V], f2[V];
#pragma unroll
    for (int j = 0; j < V; ++j) u1[j] = u2[j] = f1[j] = f2[j] = 0.f;
    float lsum = 0.f;
    for (int qq = 0; qq < NQ; ++qq) {
        cp_async_wait<BLG_R - 2>();  // this thread's copies of row qq have landed
        __syncwarp();                // ... and every lane's
        const float* cur = ring + (qq & (BLG_R - 1)) * BLG_ROW;
        const float4 u0v = *reinterpret_cast<const float4*>(cur + 4 + V * lane);
        const float u0[V] = {u0v.x, u0v.y, u0v.z, u0v.w};
        // Extra column of row r-1 (lanes 0, 31), from the previous slot.
        const float e1 = xl ? ring[((qq - 1) & (BLG_R - 1)) * BLG_ROW + xe] : 0.f;
        __syncwarp();     // the previous slot is read: refill it
        issue(qq + BLG_R - 1);
        const int r = a0 - 2 + qq;
        // x-neighbours of row r-1 at the lane's end columns.
        float um0 = __shfl_up_sync(0xffffffffu, u1[V - 1], 1);
        float upv = __shfl_down_sync(0xffffffffu, u1[0], 1);
        if (lane == 0) um0 = e1;
        if (lane == 31) upv = e1;
        if (qq >= 2) {
            float f0[V];
            if (r < nt) {
                if (r >= 2 && !gen) {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const float um = j == 0 ? um0 : u1[j - 1];
                        const float up = j == V - 1 ? upv : u1[j + 1];
                        f0[j] = blg_f(g, u0[j], u1[j], u2[j], um, up);
                    }
                    if (fixm) {
                        // Columns 0 / nx - 1: the extrapolated neighbour of
                        // wave_f_with from the streamed boundary value.
#pragma unroll
                        for (int j = 0; j < V; ++j) {
                            if (fixm & (1u << j)) {
                                float um = j == 0 ? um0 : u1[j - 1];
                                float up = j == V - 1 ? upv : u1[j + 1];
                                if (cb + j == 0) {
                                    um = (up - 6.f * u1[j] + 8.f * cur[133]) / 3.f;
                                } else {
                                    up = (um - 6.f * u1[j] + 8.f * cur[134]) / 3.f;
                                }
                                f0[j] = blg_f(g, u0[j], u1[j], u2[j], um, up);
                            }
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const float um = j == 0 ? um0 : u1[j - 1];
                        const float up = j == V - 1 ? upv : u1[j + 1];
                        f0[j] = wave_f(g, r, off[j], u0[j], u1[j], u2[j], um, up);
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < V; ++j) f0[j] = 0.f;
            }
            // Gradient of row a = r - 2 from f rows a, a+1 (with its
            // x-neighbours) and a+2.
            const int a = r - 2;
            if (qq >= 4 && a < nt) {
                const float fm0 = __shfl_up_sync(0xffffffffu, f1[V - 1], 1);
                const float fpv = __shfl_down_sync(0xffffffffu, f1[0], 1);
                float gv[V];
                if (a >= 1 && a + 2 < nt && !gen) {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const float f1m = j == 0 ? fm0 : f1[j - 1];
                        const float f1p = j == V - 1 ? fpv : f1[j + 1];
                        gv[j] = A * (f2[j] + f0[j]) + ctm[j] * f1[j] -
                                B * (kxm1[j] * f1p + kxp1[j] * f1m);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const float f1m = j == 0 ? fm0 : f1[j - 1];
                        const float f1p = j == V - 1 ? fpv : f1[j + 1];
                        gv[j] = wave_gather(g, a, off[j], f2[j], f1[j], f0[j], f1p, f1m);
                    }
                }
                float* __restrict__ grow = gi + (int64_t)a * nx + cb;
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    if (outm & (1u << j)) {
                        grow[j] = gv[j] * gscale;
                        lsum += f2[j] * f2[j];
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < V; ++j) {
                f2[j] = f1[j];
                f1[j] = f0[j];
            }
        }
#pragma unroll
        for (int j = 0; j < V; ++j) {
            u2[j] = u1[j];
            u1[j] = u0[j];
        }
    }
    cp_async_wait<0>();
    // The warp's 32 lane sums in FP32 (shuffles; GB300's FP64 pipe is
    // narrow), the item's partial in FP64.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) partials[item] = (double)lsum;
}

// loss[i] = (sum of instance i's block sums) / N_i, one warp per instance
// (lane-strided, fixed tree: deterministic).
__global__ void __launch_bounds__(256) batch_loss_finish_kernel(
    const odil_wave_instance* __restrict__ inst, int ninst,
    const int64_t* __restrict__ tile_start, const double* __restrict__ partials,
    double* __restrict__ loss) {
    const int q = (int)(((int64_t)blockIdx.x * 256 + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (q >= ninst) return;
    const int64_t a = tile_start[q], b = tile_start[q + 1];
    double s = 0.0;
    for (int64_t k = a + lane; k < b; k += 32) s += __ldcg(partials + k);
    s = warp_sum(s);
    if (lane == 0) loss[q] = s / ((double)inst[q].nt * (double)inst[q].nx);
}

// total = sum_i loss[i] in a fixed order (one block).
__global__ void __launch_bounds__(256) batch_loss_total_kernel(const double* __restrict__ loss,
                                                               int ninst,
                                                               double* __restrict__ total) {
    const double t = sum_partials(loss, ninst);
    if (threadIdx.x == 0) total[0] = t;
}

}  // namespace
}  // namespace odil

using namespace odil;

ODIL_API int odil_wave_batch_loss_grad_f32(const odil_wave_batch* b, const int64_t* tile_start,
                                           const int32_t* tile_inst, int64_t ntiles,
                                           const float* init_u,
                                           const float* init_ut, const float* left_u,
                                           const float* right_u, const float* u, float* grad,
                                           double* partials, double* loss, double* total,
                                           void* stream) {
    int st = check_batch(b);
    if (st) return st;
    if (ntiles < 1 || ntiles > (int64_t)1 << 31) return ODIL_ERR_SHAPE;
    if (!tile_start || !tile_inst || !init_u || !init_ut || !left_u || !right_u || !u || !grad ||
        !partials || !loss)
        return ODIL_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    batch_loss_grad_kernel<<<(unsigned)((ntiles + BLG_WARPS - 1) / BLG_WARPS), BLG_WARPS * 32, 0,
                             s>>>(b->inst, tile_inst, tile_start, ntiles, init_u, init_ut, left_u,
                                  right_u, u, grad, partials);
    batch_loss_finish_kernel<<<(unsigned)((b->ninst * 32 + 255) / 256), 256, 0, s>>>(
        b->inst, b->ninst, tile_start, partials, loss);
    if (total) batch_loss_total_kernel<<<1, 256, 0, s>>>(loss, b->ninst, total);
    return launch_status();
}

ODIL_API int64_t odil_wave_batch_loss_grad_items(int64_t nt, int64_t nx) {
    if (nt < 1 || nx < 1) return ODIL_ERR_SHAPE;
    return ((nx + BLG_OUT - 1) / BLG_OUT) * ((nt + BLG_TY - 1) / BLG_TY);
}

ODIL_API int odil_wave_batch_setup(odil_wave_instance* inst, int32_t ninst, void* stream) {
    if (!inst || ninst < 1) return ODIL_ERR_ARG;
    batch_setup_kernel<<<(ninst + 127) / 128, 128, 0, as_stream(stream)>>>(inst, ninst);
    return launch_status();
}

ODIL_API int64_t odil_wave_batch_workspace_bytes(const odil_wave_batch* b) {
    (void)b;
    return 256;
}

ODIL_API int odil_wave_batch_update_residual_mixed(const odil_wave_batch* b, const double* u,
                                                   const float* d, double* u_out, float* rhs,
                                                   void* stream) {
    int st = check_batch(b);
    if (st) return st;
    if (!u || !rhs || (d && (!u_out || u_out == u))) return ODIL_ERR_ARG;
    if (!b->init_u || !b->init_ut || !b->left_u || !b->right_u) return ODIL_ERR_ARG;
    int64_t blocks = (b->total_cells + 255) / 256;
    const int64_t cap = (int64_t)sms() * 16;
    if (blocks > cap) blocks = cap;
    batch_update_residual_kernel<<<(int)blocks, 256, 0, as_stream(stream)>>>(*b, u, d, u_out,
                                                                             rhs);
    return launch_status();
}

ODIL_API int odil_wave_batch_initial_rhs_mixed(const odil_wave_batch* b, float* rhs,
                                               void* stream) {
    int st = check_batch(b);
    if (st) return st;
    if (!rhs) return ODIL_ERR_ARG;
    if (!b->init_u || !b->init_ut || !b->left_u || !b->right_u) return ODIL_ERR_ARG;
    return launch_rhs<0>(b, nullptr, nullptr, rhs, as_stream(stream));
}

ODIL_API int odil_wave_batch_pair_residual_mixed(const odil_wave_batch* b, const float* hi,
                                                 const float* lo, float* rhs, void* stream) {
    int st = check_batch(b);
    if (st) return st;
    if (!hi || !rhs || rhs == hi || rhs == lo) return ODIL_ERR_ARG;
    if (!b->init_u || !b->init_ut || !b->left_u || !b->right_u) return ODIL_ERR_ARG;
    return launch_rhs<1>(b, hi, lo, rhs, as_stream(stream));
}

ODIL_API int odil_wave_batch_solve_mixed(const odil_wave_batch* b, int32_t epochs, float* rhs,
                                         float* hi, float* lo, double* u,
                                         int32_t threads, int32_t cpt, int32_t pf,
                                         int32_t blocks_per_sm, void* workspace,
                                         int64_t workspace_bytes, void* stream) {
    int st = check_batch(b);
    if (st) return st;
    if (epochs < 1 || epochs > 16) return ODIL_ERR_ARG;
    if (!rhs || !hi || !u || (epochs > 1 && !lo)) return ODIL_ERR_ARG;
    if (!b->init_u || !b->init_ut || !b->left_u || !b->right_u) return ODIL_ERR_ARG;
    if (!workspace || workspace_bytes < 256) return ODIL_ERR_WORKSPACE;
    if (threads < 32 || threads > 1024 || threads % 32 || blocks_per_sm < 1 || blocks_per_sm > 32)
        return ODIL_ERR_SHAPE;
    int blocks = sms() * blocks_per_sm;
    if (blocks > b->ninst) blocks = b->ninst;
    unsigned* counter = reinterpret_cast<unsigned*>(workspace);
    cudaStream_t s = as_stream(stream);
    switch (cpt * 100 + pf) {
        case 108: return launch_batch_solve<1, 8>(b, epochs, rhs, hi, lo, u, counter, threads, blocks, s);
        case 116: return launch_batch_solve<1, 16>(b, epochs, rhs, hi, lo, u, counter, threads, blocks, s);
        case 208: return launch_batch_solve<2, 8>(b, epochs, rhs, hi, lo, u, counter, threads, blocks, s);
        case 408: return launch_batch_solve<4, 8>(b, epochs, rhs, hi, lo, u, counter, threads, blocks, s);
        default: return ODIL_ERR_SHAPE;
    }
}

ODIL_API int odil_wave_batch_march_f32(const odil_wave_batch* b, const float* rhs, float* x,
                                       int32_t threads, int32_t cpt, int32_t pf,
                                       int32_t blocks_per_sm, void* workspace,
                                       int64_t workspace_bytes, void* stream) {
    int st = check_batch(b);
    if (st) return st;
    if (!rhs || !x) return ODIL_ERR_ARG;
    if (!workspace || workspace_bytes < 256) return ODIL_ERR_WORKSPACE;
    if (threads < 32 || threads > 1024 || threads % 32 || blocks_per_sm < 1 || blocks_per_sm > 32)
        return ODIL_ERR_SHAPE;
    int blocks = sms() * blocks_per_sm;
    if (blocks > b->ninst) blocks = b->ninst;
    unsigned* counter = reinterpret_cast<unsigned*>(workspace);
    cudaStream_t s = as_stream(stream);
    const int key = cpt * 100 + pf;
    switch (key) {
        case 108: return launch_batch_march<1, 8>(b, rhs, x, counter, threads, blocks, s);
        case 116: return launch_batch_march<1, 16>(b, rhs, x, counter, threads, blocks, s);
        case 208: return launch_batch_march<2, 8>(b, rhs, x, counter, threads, blocks, s);
        case 216: return launch_batch_march<2, 16>(b, rhs, x, counter, threads, blocks, s);
        case 408: return launch_batch_march<4, 8>(b, rhs, x, counter, threads, blocks, s);
        case 416: return launch_batch_march<4, 16>(b, rhs, x, counter, threads, blocks, s);
        default: return ODIL_ERR_SHAPE;
    }
}
