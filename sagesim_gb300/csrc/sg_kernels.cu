// sg_kernels.cu -- pull-strategy, frontier-strategy and opinion tick kernels
// for sm_103a, and the CSR utilities (placement offsets, transpose).
//
// The tick semantics follow SAGESim's generated fused kernel
// (sagesim/model.py:2306-2408): every step reads tick-start values and writes a
// separate buffer; the next tick reads what this tick wrote. Here the two
// buffers ping-pong (buffer (par0 + r) & 1 is read at relative tick r), so the
// reference's per-tick write-back copy (model.py:2374-2389) disappears.
//
// Work decomposition: a persistent grid walks a tile list (tiles never straddle
// segments). Rows are binned by length: a lane scans a row of up to thread_row
// entries, a warp a row of up to mega_row entries, and rows longer than that
// are listed at setup and scanned by dedicated blocks. The count strategy's
// kernels are in sg_count.cu.
#include <cub/device/device_scan.cuh>

#include <mutex>

#include "sg_device.cuh"

namespace {

// ---- pull strategy --------------------------------------------------------------
// Blocks [0, gridDim.x - a.mega_blocks) walk the tiles, one warp per 32
// consecutive agents; the last a.mega_blocks blocks each take mega rows.
template <int VARIANT, bool STATS>
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_pull_kernel(SgTickArgs a)
{
    __shared__ unsigned long long red[4][kWarps];
    __shared__ int32_t sh_count;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int32_t *__restrict__ off = a.off;
    const int32_t *__restrict__ idx = a.idx;
    const int tile_blocks = (int)gridDim.x - a.mega_blocks;

    if ((int)blockIdx.x >= tile_blocks) {
        for (int q = (int)blockIdx.x - tile_blocks; q < a.nmega; q += a.mega_blocks) {
            const SgMega mg = a.mega[q];
            const SgSeg &sg = a.segs[mg.seg];
            const int64_t tick = sg.tick0 + a.r;
            if (tick >= sg.end_tick) continue;
            const int par = (sg.par0 + a.r) & 1;
            const int32_t *__restrict__ sin = (const int32_t *)(par ? a.buf1 : a.buf0);
            int32_t *__restrict__ sout = (int32_t *)(par ? a.buf0 : a.buf1);
            const int32_t h = mg.agent;
            if (sin[h] != sg.cs) continue; // handled by the tile pass
            const uint32_t c0b = sg_c0base(tick);
            const uint32_t lid = seg_lid(sg, h);
            bool lucky = true;
            if (VARIANT == 1) lucky = sg_philox_k23(c0b + 1u, lid, sg.key) < sg.kinf;
            bool inf = false;
            if (lucky)
                inf = block_row<VARIANT>(idx, sin, __ldg(off + h), __ldg(off + h + 1), sg.ci, c0b,
                                         lid, sg.key, sg.kinf, &sh_count, nullptr);
            if (tid == 0) {
                sout[h] = inf ? sg.ci : sg.cs;
                if (STATS && sg.stats) {
                    atomicAdd(sg.stats + 4 * (int64_t)a.r + (inf ? 1 : 0), 1ull);
                    atomicAdd(sg.stats + 4 * (int64_t)a.r + 3,
                              (unsigned long long)(__ldg(off + h + 1) - __ldg(off + h)));
                }
            }
        }
        return;
    }

    for (int t = blockIdx.x; t < a.ntiles; t += tile_blocks) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int64_t tick = sg.tick0 + a.r;
        if (tick >= sg.end_tick) continue; // uniform over the block
        const int par = (sg.par0 + a.r) & 1;
        const int32_t *__restrict__ sin = (const int32_t *)(par ? a.buf1 : a.buf0);
        int32_t *__restrict__ sout = (int32_t *)(par ? a.buf0 : a.buf1);
        const uint32_t c0b = sg_c0base(tick);
        const uint32_t key = sg.key, kinf = sg.kinf, krec = sg.krec;
        const int32_t cs = sg.cs, ci = sg.ci, cr = sg.cr;
        const int32_t mega_row = a.mega_row;
        const int32_t thread_row = thread_row_of(a);
        unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;

        for (int32_t wbase = tile.begin + warp * 32; wbase < tile.end; wbase += SG_SIR_THREADS) {
            const int32_t i = wbase + lane;
            const bool valid = i < tile.end;
            const int32_t s = valid ? sin[i] : INT32_MIN;
            int32_t out = s;
            bool medium = false, skip = false;
            int32_t b = 0, e = 0;
            uint32_t lid = 0;
            if (s == ci) {
                if (sg_philox_k23(c0b + 1u, seg_lid(sg, i), key) < krec) out = cr;
            } else if (s == cs) {
                lid = seg_lid(sg, i);
                const bool lucky = VARIANT == 2 || sg_philox_k23(c0b + 1u, lid, key) < kinf;
                if (lucky || STATS) {
                    b = __ldg(off + i);
                    e = __ldg(off + i + 1);
                    if (e - b > mega_row) {
                        skip = true; // a mega block writes this agent
                    } else {
                        if (STATS) eS += (unsigned long long)(e - b);
                        if (lucky) {
                            if (e - b > thread_row)
                                medium = true;
                            else if (VARIANT == 1 ? any_infected_thread(idx, sin, b, e, ci)
                                                  : trials_thread(idx, sin, b, e, ci, c0b, lid, key,
                                                                  kinf))
                                out = ci;
                        }
                    }
                }
            }
            unsigned m = __ballot_sync(FULL_MASK, medium);
            while (m) {
                const int l = __ffs(m) - 1;
                m &= m - 1;
                const int32_t hb = __shfl_sync(FULL_MASK, b, l);
                const int32_t he = __shfl_sync(FULL_MASK, e, l);
                const uint32_t hl = __shfl_sync(FULL_MASK, lid, l);
                const bool inf = warp_row<VARIANT>(idx, sin, hb, he, ci, c0b, hl, key, kinf, lane,
                                                   nullptr);
                if (lane == l && inf) out = ci;
            }
            if (valid && !skip) {
                sout[i] = out;
                if (STATS) {
                    nS += (out == cs);
                    nI += (out == ci);
                    nR += (out == cr);
                }
            }
        }
        if (STATS && sg.stats) block_flush4(nS, nI, nR, eS, sg.stats + 4 * (int64_t)a.r, red);
    }
}

// ---- frontier strategy ------------------------------------------------------------
// Only "active" agents can change: infected agents (recovery draw) and
// susceptible agents with at least one infected neighbour (cnt > 0). The
// frontier strategy keeps them in a compact list per tick, so a tick costs
// O(active + edges of changed agents) instead of O(agents):
//   build  (run start) list[0] = {I} U {S with cnt > 0}; mark[i] = 0 for them
//   step r   each listed agent draws; it stays listed (mark = r+1, appended to
//            list r+1) while it is I or S with cnt > 0; S->I and I->R changes go
//            to the change list of tick r
//   scatter r  +-1 along the transpose rows of the changes; a susceptible agent
//            whose count goes 0 -> 1 joins list r+1 unless mark[] says it is
//            already there (atomicExch on mark deduplicates)
// State is updated in place (only listed agents are touched), and the draws
// are the same as in the count strategy, so results are bit-identical.

// All threads of the block call it: appends `value` for every thread whose
// flag is set, one global atomic per block.
__device__ __forceinline__ void block_append(bool flag, int32_t value, int32_t *__restrict__ list,
                                             int32_t *counter, int32_t *sh /* kWarps + 1 */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(FULL_MASK, flag);
    if (lane == 0) sh[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t total = 0;
        for (int w = 0; w < kWarps; ++w) {
            const int32_t c = sh[w];
            sh[w] = total;
            total += c;
        }
        sh[kWarps] = total ? atomicAdd(counter, total) : 0;
    }
    __syncthreads();
    if (flag) list[sh[kWarps] + sh[warp] + __popc(m & ((1u << lane) - 1u))] = value;
    __syncthreads();
}

__device__ __forceinline__ const SgSeg &seg_of(const SgTickArgs &a, int32_t agent)
{
    return a.segs[a.aseg ? __ldg(a.aseg + agent) : 0];
}

// list[0] and mark[] from the tiles; with STATS also the initial S/I/R/E_S totals.
template <bool STATS>
__global__ void __launch_bounds__(SG_SIR_THREADS) frontier_build_kernel(SgTickArgs a)
{
    __shared__ int32_t sh[kWarps + 1];
    __shared__ unsigned long long red[4][kWarps];
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int32_t *st = (const int32_t *)a.buf0;
        unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;
        for (int32_t base = tile.begin; base < tile.end; base += SG_SIR_THREADS) {
            const int32_t i = base + tid;
            bool in = false;
            if (i < tile.end) {
                const int32_t s = st[i];
                in = (s == sg.ci) || (s == sg.cs && a.cnt[i] > 0);
                a.mark[i] = in ? 0 : -1;
                if (STATS) {
                    nS += (s == sg.cs);
                    nI += (s == sg.ci);
                    nR += (s == sg.cr);
                    if (s == sg.cs) eS += (unsigned long long)(a.off[i + 1] - a.off[i]);
                }
            }
            block_append(in, i, a.list[0], a.list_len, sh);
        }
        if (STATS && sg.stats) block_flush4(nS, nI, nR, eS, a.stats_init, red);
    }
}

// STATS rows are deltas: infections, recoveries, sum of the infected agents'
// degrees (the engine turns them into absolute S/I/R/E_S per tick).
template <int VARIANT, bool STATS>
__global__ void __launch_bounds__(SG_SIR_THREADS) frontier_step_kernel(SgTickArgs a)
{
    __shared__ int32_t sh[kWarps + 1];
    __shared__ unsigned long long red[4][kWarps];
    constexpr int U = 4;
    const int tid = threadIdx.x;
    const int32_t n = a.list_len[a.r];
    const int32_t *__restrict__ lin = a.list[a.r & 1];
    int32_t *__restrict__ lout = a.list[(a.r + 1) & 1];
    int32_t *st = (int32_t *)a.buf0;
    unsigned long long dInf = 0, dRec = 0, dDeg = 0;
    for (int32_t base = blockIdx.x * (SG_SIR_THREADS * U); base < n; base += gridDim.x * (SG_SIR_THREADS * U)) {
        int32_t ag[U], s[U], k[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int32_t q = base + u * SG_SIR_THREADS + tid;
            ag[u] = q < n ? lin[q] : -1;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) s[u] = ag[u] >= 0 ? st[ag[u]] : INT32_MIN;
#pragma unroll
        for (int u = 0; u < U; ++u) k[u] = ag[u] >= 0 ? a.cnt[ag[u]] : 0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            bool keep = false, chg = false, sus = false;
            int32_t code = 0, sci = 0;
            uint32_t slid = 0, sc0b = 0, skey = 0, skinf = 0;
            if (ag[u] >= 0) {
                const int32_t i = ag[u];
                const SgSeg &sg = seg_of(a, i);
                const int64_t tick = sg.tick0 + a.r;
                if (tick < sg.end_tick) {
                    const uint32_t c0b = sg_c0base(tick);
                    if (s[u] == sg.ci) {
                        if (sg_philox_k23(c0b + 1u, seg_lid(sg, i), sg.key) < sg.krec) {
                            st[i] = sg.cr;
                            chg = true;
                            code = ~i;
                            if (STATS) ++dRec;
                        } else {
                            keep = true;
                        }
                    } else if (s[u] == sg.cs && k[u] > 0) {
                        sus = true;
                        keep = true;
                        slid = seg_lid(sg, i);
                        sc0b = c0b;
                        skey = sg.key;
                        skinf = sg.kinf;
                        sci = sg.ci;
                    }
                    if (keep) a.mark[i] = a.r + 1;
                }
            }
            // susceptible agents with infected neighbours: the draws
            bool inf;
            if (VARIANT == 1)
                inf = sus && sg_philox_k23(sc0b + 1u, slid, skey) < skinf;
            else
                inf = sirb_infected(sus, k[u], sc0b, slid, skey, skinf, tid & 31);
            if (inf) {
                const int32_t i = ag[u];
                st[i] = sci;
                chg = true;
                code = i;
                if (STATS) {
                    ++dInf;
                    dDeg += (unsigned long long)(a.off[i + 1] - a.off[i]);
                }
            }
            block_append(keep, ag[u], lout, a.list_len + a.r + 1, sh);
            block_append(chg, code, a.changes, a.nch + a.r, sh);
        }
    }
    if (STATS && a.stats_delta) block_flush4(dInf, dRec, dDeg, 0ull, a.stats_delta + 4 * (int64_t)a.r, red);
}

__global__ void __launch_bounds__(SG_SIR_THREADS) frontier_scatter_kernel(SgTickArgs a)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int32_t n = a.nch[a.r];
    const int32_t *st = (const int32_t *)a.buf0;
    int32_t *lout = a.list[(a.r + 1) & 1];
    int32_t *len = a.list_len + a.r + 1;
    const int32_t next = a.r + 1;
    const int32_t trow = thread_row_of(a);
    for (int32_t q0 = (blockIdx.x * kWarps + warp) * 32; q0 < n; q0 += gridDim.x * kWarps * 32) {
        const int32_t q = q0 + lane;
        const bool valid = q < n;
        const int32_t c = valid ? a.changes[q] : 0;
        const int32_t g = c >= 0 ? c : ~c;
        const int32_t delta = c >= 0 ? 1 : -1;
        int32_t b = 0, e = 0, cs = 0;
        if (valid) {
            b = __ldg(a.toff + g);
            e = __ldg(a.toff + g + 1);
            cs = seg_of(a, g).cs;
        }
        const bool long_row = e - b > trow;
        // candidates (count 0 -> 1, susceptible, not yet listed) are appended
        // warp-aggregated after each batch of neighbour updates
        for (int32_t t = 0;; ++t) { // row position t of every short row, in lockstep
            const bool act = !long_row && b + t < e;
            if (!__any_sync(FULL_MASK, act)) break;
            bool cand = false;
            int32_t p = 0;
            if (act) {
                p = __ldg(a.tidx + b + t);
                if (delta < 0)
                    atomicSub(a.cnt + p, 1);
                else
                    cand = atomicAdd(a.cnt + p, 1) == 0 && st[p] == cs &&
                           atomicExch(a.mark + p, next) != next;
            }
            const unsigned cm = __ballot_sync(FULL_MASK, cand);
            if (cm) {
                const int leader = __ffs(cm) - 1;
                int32_t pos = 0;
                if (lane == leader) pos = atomicAdd(len, __popc(cm));
                pos = __shfl_sync(FULL_MASK, pos, leader);
                if (cand) lout[pos + __popc(cm & ((1u << lane) - 1u))] = p;
            }
        }
        unsigned m = __ballot_sync(FULL_MASK, long_row);
        while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1;
            const int32_t hb = __shfl_sync(FULL_MASK, b, l);
            const int32_t he = __shfl_sync(FULL_MASK, e, l);
            const int32_t hd = __shfl_sync(FULL_MASK, delta, l);
            const int32_t hcs = __shfl_sync(FULL_MASK, cs, l);
            for (int32_t k0 = hb; k0 < he; k0 += 32) {
                const int32_t k = k0 + lane;
                bool cand = false;
                int32_t p = 0;
                if (k < he) {
                    p = __ldg(a.tidx + k);
                    if (hd < 0)
                        atomicSub(a.cnt + p, 1);
                    else
                        cand = atomicAdd(a.cnt + p, 1) == 0 && st[p] == hcs &&
                               atomicExch(a.mark + p, next) != next;
                }
                const unsigned cm = __ballot_sync(FULL_MASK, cand);
                if (cm) {
                    const int leader = __ffs(cm) - 1;
                    int32_t pos = 0;
                    if (lane == leader) pos = atomicAdd(len, __popc(cm));
                    pos = __shfl_sync(FULL_MASK, pos, leader);
                    if (cand) lout[pos + __popc(cm & ((1u << lane) - 1u))] = p;
                }
            }
        }
    }
}

// ---- opinion model --------------------------------------------------------------
// x' = clamp((double)(sum_j w_j x_nbr_j / sum_j |w_j|) + sigma * N(0,1), 0, 1)
// over the first min(deg, width) ordered neighbours; float32 sums in row order
// with every multiply and add rounded (no FMA), Box-Muller in double
// (sagesim/math_utils.py:231-255: u1 salt 1, u2 salt 1 + 73856093, +1e-10
// guard). u1 and u2 are k / 2^23 for 23-bit Philox integers k.
//  - radius sqrt(-2 log(u1 + 1e-10)) takes 2^23 values: it is evaluated once
//    per engine in double (opinion_tables_kernel) and tabulated twice: as the
//    correction to a float32 estimate the step recomputes (bm_radius_estimate;
//    the difference in 32-bit fixed point, steps of 2^-40: 32 MiB, kept in L2
//    as persisting lines, one 4-byte read per agent) and as double-float
//    pairs (64 MiB, in DRAM; read only for results whose rounding the first
//    form leaves open, see opinion_noise_try);
//  - cos(2 pi u2) by the angle-addition formula cos(A + B) = cos A cos B -
//    sin A sin B with k = 2048 kh + kl, A = 2 pi kh / 2^12, B = 2 pi kl / 2^23:
//    cos A from a 4096-entry table (sin A is the same table a quarter turn
//    back), cos B and sin B from 2048-entry tables (built with sincospi and
//    copied into shared memory by every block);
//  - every table entry is a double-float pair (hi, lo) of float32 whose sum is
//    the double value to about 2^-48 relative, and the noise term
//    sigma * radius * cosine and its sum with the float32 mean are formed in
//    double-float arithmetic on the FP32 units (Dekker's exact product via
//    fused multiply-add and Knuth's two-sum). This GPU's FP64 units run at a
//    small fraction of its FP32 rate; with double arithmetic they bounded the
//    tick. The result rounds to the same float32 as the reference's double
//    expression except within about 2^-46 of a float32 rounding boundary
//    (one float32 ulp apart there); the tests compare with the oracle at 1e-6
//    relative and check the cosine against the device's own cos.
// (A float32 Box-Muller was tried and rejected: opinions near the clamp at 0
// differ by up to 1.5e-4 relative.)
constexpr int32_t kBoxMullerSize = 1 << 23;
constexpr double kRadiusStep = 1099511627776.0; // 2^40: steps of the radius correction per unit

// A float32 estimate of the radius of the 23-bit integer k: sqrt(-2 ln(2)
// log2(k 2^-23 + 1e-10)) with the hardware's approximate base-2 logarithm and a
// correctly rounded square root, clamped at 0. Each operation is an explicitly
// rounded intrinsic or that logarithm, so every kernel computes the same value
// and the table's correction is the one for the step's estimate. The error is
// largest near k = 2^23, where -log u is tiny and the logarithm's absolute
// error (about 2^-22) dominates: up to the square root of that, about 2^-10.5;
// far smaller elsewhere. The corrections' range (2^-9) covers it.
__device__ __forceinline__ float bm_radius_estimate(uint32_t k)
{
    const float u = __fadd_rn(__fmul_rn(__uint2float_rn(k), 0x1p-23f), 1e-10f);
    const float l = __fmul_rn(-1.38629436f, __log2f(u)); // -2 ln(2) log2(u)
    return __fsqrt_rn(fmaxf(l, 0.0f));
}
constexpr int32_t kTrigA = 4096, kTrigB = 2048; // entries of the A (cos) and B (cos, sin) tables
static_assert(kTrigA + 2 * kTrigB == SG_BM_TRIG_ENTRIES, "table layout");

__device__ __forceinline__ double bm_radius(uint32_t k)
{
    const double u1 = (double)k / 8388608.0;
    return sqrt(__dmul_rn(-2.0, log(__dadd_rn(u1, 1e-10))));
}

__device__ __forceinline__ double bm_cos(uint32_t k)
{
    const double u2 = (double)k / 8388608.0;
    return cos(__dmul_rn(6.283185307179586, u2));
}

// ---- double-float arithmetic (hi + lo, |lo| <= ulp(hi) / 2) ----
__device__ __forceinline__ float2 ff_split(double v)
{
    const float hi = __double2float_rn(v);
    return make_float2(hi, __double2float_rn(v - (double)hi));
}

// a + b exactly as s + e (Knuth's two-sum; any magnitudes)
__device__ __forceinline__ float2 ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}

// s + e renormalised when |s| >= |e| (fast two-sum)
__device__ __forceinline__ float2 ff_norm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}

// a * b: exact product of the high parts (Dekker, via fma) plus the cross terms
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return ff_norm(p, e);
}

// a + b
__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    float2 s = ff_two_sum(a.x, b.x);
    const float2 t = ff_two_sum(a.y, b.y);
    s = ff_norm(s.x, __fadd_rn(s.y, t.x));
    return ff_norm(s.x, __fadd_rn(s.y, t.y));
}

// trig = [cos A (4096)][cos B (2048)][sin B (2048)] as double-float pairs, in
// global or shared memory
__device__ __forceinline__ float2 bm_cos_split(const float2 *trig, uint32_t k)
{
    const uint32_t kh = k >> 11, kl = k & (kTrigB - 1);
    const float2 ca = trig[kh], sa = trig[(kh - kTrigA / 4) & (kTrigA - 1)]; // sin A = cos(A - pi/2)
    const float2 cb = trig[kTrigA + kl], sb = trig[kTrigA + kTrigB + kl];
    const float2 p = ff_mul(sa, sb);
    return ff_add(ff_mul(ca, cb), make_float2(-p.x, -p.y));
}

__global__ void opinion_tables_kernel(float2 *__restrict__ radius, uint32_t *__restrict__ rq,
                                      float2 *__restrict__ trig)
{
    const int32_t stride = gridDim.x * blockDim.x;
    const int32_t end = radius ? kBoxMullerSize : kTrigA; // radius NULL: the cosine tables only
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < end; k += stride) {
        if (radius) {
            const double rv = bm_radius((uint32_t)k);
            radius[k] = ff_split(rv);
            if (rq) { // the difference (exact in double) in steps of 2^-40
                const double d = rv - (double)bm_radius_estimate((uint32_t)k);
                rq[k] = (uint32_t)__double2int_rn(d * kRadiusStep);
            }
        }
        if (k < kTrigA) { // A = pi * k / 2^11
            double sv, cv;
            sincospi((double)k / 2048.0, &sv, &cv);
            trig[k] = ff_split(cv);
        }
        if (k < kTrigB) { // B = pi * k / 2^22
            double sv, cv;
            sincospi((double)k / 4194304.0, &sv, &cv);
            trig[kTrigA + k] = ff_split(cv);
            trig[kTrigA + kTrigB + k] = ff_split(sv);
        }
    }
}

// First 8 neighbours of every agent, group-major (SG_NB8_AT), -1 after the row
// ends and for the agents >= n of the last group.
__global__ void opinion_neighbours8_kernel(const int32_t *__restrict__ off, const int32_t *__restrict__ idx,
                                           int64_t n, int32_t *__restrict__ nb8)
{
    const int64_t nall = (n + 31) & ~(int64_t)31;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nall; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t b = 0, m = 0;
        if (i < n) {
            b = off[i];
            m = min(off[i + 1] - b, 8);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) nb8[SG_NB8_AT(i, j)] = j < m ? idx[b + j] : -1;
    }
}

// Cosine by the split tables for k0 <= k < k0 + n (the tests compare it with
// cos(2 pi k / 2^23) evaluated directly).
__global__ void opinion_cos_check_kernel(const float2 *__restrict__ trig, int32_t k0, int32_t n, double *out)
{
    for (int32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)(k0 + q);
        const float2 c = bm_cos_split(trig, k);
        out[2 * q] = (double)c.x + (double)c.y;
        out[2 * q + 1] = bm_cos(k);
    }
}

// All of a row's loads are issued before the sums: for width 8 the weight row
// is two 16-byte loads, then the (up to 8) neighbour indices, then their opinions.
template <int W> // 8, or 0 for any width
__device__ __forceinline__ float opinion_mean(const SgTickArgs &a, const SgSeg &sg, const float *__restrict__ xin,
                                              int32_t i, int32_t width)
{
    const int32_t b = __ldg(a.off + i);
    int32_t m = __ldg(a.off + i + 1) - b;
    if (m > width) m = width;
    float acc = 0.0f, norm = 0.0f;
    if (W == 8) {
        // weights, row indices and the Box-Muller tables are read once per tick:
        // evict-first loads keep L2 for the opinions, which neighbours re-read
        const float4 *w4 = reinterpret_cast<const float4 *>(sg.weights + (int64_t)i * 8);
        const float4 w0 = __ldcs(w4), w1 = __ldcs(w4 + 1);
        const float wv[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
        // the row's first 8 indices: vector loads when the row start allows
        // (a warp's rows are contiguous, so each load instruction is dense)
        int32_t nb[8];
        if (m == 8 && (b & 3) == 0) {
            const int4 *p4 = reinterpret_cast<const int4 *>(a.idx + b);
            const int4 v0 = __ldcs(p4), v1 = __ldcs(p4 + 1);
            nb[0] = v0.x, nb[1] = v0.y, nb[2] = v0.z, nb[3] = v0.w, nb[4] = v1.x, nb[5] = v1.y, nb[6] = v1.z, nb[7] = v1.w;
        } else if (m == 8 && (b & 1) == 0) {
            const int2 *p2 = reinterpret_cast<const int2 *>(a.idx + b);
            const int2 v0 = __ldcs(p2), v1 = __ldcs(p2 + 1), v2 = __ldcs(p2 + 2), v3 = __ldcs(p2 + 3);
            nb[0] = v0.x, nb[1] = v0.y, nb[2] = v1.x, nb[3] = v1.y, nb[4] = v2.x, nb[5] = v2.y, nb[6] = v3.x, nb[7] = v3.y;
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) nb[j] = j < m ? __ldcs(a.idx + b + j) : i;
        }
        float xv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) xv[j] = __ldg(xin + nb[j]);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (j < m) {
                acc = __fadd_rn(acc, __fmul_rn(wv[j], xv[j]));
                norm = __fadd_rn(norm, fabsf(wv[j]));
            }
    } else {
        const float *__restrict__ w = sg.weights + (int64_t)i * width;
        for (int32_t j = 0; j < m; ++j) {
            const float wj = __ldg(w + j);
            const float xj = __ldg(xin + __ldg(a.idx + b + j));
            acc = __fadd_rn(acc, __fmul_rn(wj, xj));
            norm = __fadd_rn(norm, fabsf(wj));
        }
    }
    return norm > 0.0f ? __fdiv_rn(acc, norm) : xin[i];
}

// Persistent blocks of kOpinionThreads threads (64 KiB of cosine tables in
// shared memory each), work handed out round robin in chunks of one agent per
// thread (any width) or, for width 8, two agents per thread: the opinion tick
// is bound by the latency of its dependent loads (row bounds, then row
// indices, then neighbour opinions), so a thread issues every load of a phase
// for both of its agents before it waits on any, and the noise draw and its
// radius load, which need no graph data, go first.
constexpr int kOpinionThreads = 512;

// Noise and clamp: y = x + sigma * radius * cos, rounded to float32 and
// clamped to [0, 1]. Rounding is monotone and keeps 0 and 1, so clamping after
// rounding gives the same value as clamping first; a negative value rounds to a
// non-positive float, stored as +0.
__device__ __forceinline__ float clamp_opinion(float y)
{
    return y <= 0.0f ? 0.0f : (y > 1.0f ? 1.0f : y);
}

// With the tables: x + sigma * r * c in double-float (r, c the radius and
// cosine pairs), rounded to float32 and clamped.
__device__ __forceinline__ float opinion_noise_pair(const SgTickArgs &a, float x, float2 r, float2 c)
{
    const float2 t = ff_mul(make_float2(a.sigma_hi, a.sigma_lo), ff_mul(r, c));
    const float2 s2 = ff_two_sum(x, t.x); // x + t, rounded once
    return clamp_opinion(ff_norm(s2.x, __fadd_rn(s2.y, t.y)).x);
}

// The same result from the estimate re of the radius of k1 and its correction
// dq (steps of 2^-40), when it can tell: y is formed as in opinion_noise_pair
// with r = re + dq 2^-40 (within 2^-41 of the double radius and 2^-40.9 of
// the pair table's), and it differs from the pair-table value by at most E =
// sigma |c| 2^-40 + 2^-42 (|t| + |y|) (that radius difference times sigma |c|,
// plus both paths' double-float roundings, each a few 2^-48 of |t| and |y|).
// When y - E and y + E round and clamp to the same float32, so does the
// pair-table value (rounding is monotone). Otherwise (near a float32 rounding
// boundary: about one draw in 10^5, most at tiny opinions, whose float32 steps
// are finest) *sure is false.
__device__ __forceinline__ float opinion_noise_try(const SgTickArgs &a, float x, float re, uint32_t dq, float2 c,
                                                   bool *sure)
{
    // re + dq 2^-40 as a pair: dq's bits above the low 8 and its low 8 convert exactly
    const float2 rh = ff_norm(re, __fmul_rn(__int2float_rn((int32_t)(dq & 0xFFFFFF00u)), 0x1p-40f));
    const float2 r = ff_norm(rh.x, __fadd_rn(rh.y, __fmul_rn(__uint2float_rn(dq & 0xFFu), 0x1p-40f)));
    const float2 t = ff_mul(make_float2(a.sigma_hi, a.sigma_lo), ff_mul(r, c));
    const float2 s2 = ff_two_sum(x, t.x);
    const float lo = __fadd_rn(s2.y, t.y);
    const float e = __fmul_rn(__fadd_rn(__fadd_rn(fabsf(t.x), fabsf(s2.x)), 4.0f * a.sigma_hi * fabsf(c.x)), 0x1p-42f);
    const float ya = clamp_opinion(__fadd_rn(s2.x, __fsub_rd(lo, e)));
    const float yb = clamp_opinion(__fadd_rn(s2.x, __fadd_ru(lo, e)));
    *sure = ya == yb;
    return ya;
}

// Noise and clamp for one agent (k1, k2 the draw's two integers, dq the radius
// correction of k1 when the tables are present): always the value of
// opinion_noise_pair with the pair-table radius, which is read only when the
// estimate and correction leave the rounding open. Without tables (no cosine
// pairs) the expression is evaluated in double.
__device__ __forceinline__ float opinion_noise(const SgTickArgs &a, const SgSeg &sg, const float2 *trig, float x,
                                               uint32_t dq, uint32_t k1, uint32_t k2)
{
    if (a.bm_rq && a.bm_radius && trig) {
        const float2 c = bm_cos_split(trig, k2);
        bool sure;
        const float y = opinion_noise_try(a, x, bm_radius_estimate(k1), dq, c, &sure);
        return sure ? y : opinion_noise_pair(a, x, __ldg(a.bm_radius + k1), c);
    }
    const double z = __dmul_rn(bm_radius(k1), bm_cos(k2));
    return clamp_opinion(__double2float_rn(__dadd_rn((double)x, __dmul_rn(sg.sigma, z))));
}

// out[q] = the step's noise result for opinion x[q] and the draw's integers
// k1[q], k2[q] (a.bm_radius, a.bm_rq, a.bm_trig and sigma set); exact[q] = the
// value with the pair-table radius; slow[q] = 1 where the fixed-point radius
// left the rounding open (q < n).
__global__ void opinion_noise_check_kernel(SgTickArgs a, const float *x, const uint32_t *k1, const uint32_t *k2,
                                           int64_t n, float *out, float *exact, uint8_t *slow)
{
    const SgSeg sg{};
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float2 c = bm_cos_split(a.bm_trig, k2[q]);
        bool sure;
        const uint32_t dq = a.bm_rq[k1[q]];
        (void)opinion_noise_try(a, x[q], bm_radius_estimate(k1[q]), dq, c, &sure);
        out[q] = opinion_noise(a, sg, a.bm_trig, x[q], dq, k1[q], k2[q]);
        exact[q] = opinion_noise_pair(a, x[q], a.bm_radius[k1[q]], c);
        slow[q] = sure ? 0 : 1;
    }
}

template <int W>
__global__ void __launch_bounds__(kOpinionThreads, W == 8 ? 2 : 3) opinion_kernel(SgTickArgs a)
{
    extern __shared__ float2 sh_trig[]; // SG_BM_TRIG_ENTRIES pairs when a.bm_trig is set
    if (a.bm_trig) {
        const float4 *src = reinterpret_cast<const float4 *>(a.bm_trig);
        for (int j = threadIdx.x; j < SG_BM_TRIG_ENTRIES / 2; j += kOpinionThreads)
            reinterpret_cast<float4 *>(sh_trig)[j] = __ldg(src + j);
        __syncthreads();
    }
    const float2 *trig = a.bm_trig ? sh_trig : nullptr;
    constexpr int32_t U = W == 8 ? 2 : 1;                      // agents per thread and chunk
    constexpr int32_t parts = SG_TILE / (kOpinionThreads * U); // chunks per tile
    const int32_t nchunks = a.ntiles * parts;
    for (int32_t q = blockIdx.x; q < nchunks; q += gridDim.x) {
        const SgTile tile = a.tiles[q / parts];
        const SgSeg &sg = a.segs[tile.seg];
        const int64_t tick = sg.tick0 + a.r;
        if (tick >= sg.end_tick) continue; // the same for the whole block
        const int par = (sg.par0 + a.r) & 1;
        const float *__restrict__ xin = (const float *)(par ? a.buf1 : a.buf0);
        float *__restrict__ xout = (float *)(par ? a.buf0 : a.buf1);
        const uint32_t c0b = sg_c0base(tick);
        int32_t iu[U];
        bool vu[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int32_t i = tile.begin + (q % parts) * (kOpinionThreads * U) + u * kOpinionThreads +
                              (int32_t)threadIdx.x;
            vu[u] = i < tile.end;
            iu[u] = vu[u] ? i : tile.begin; // a valid agent keeps every load in bounds
        }
        // 1. the normal draw's two Philox integers and the radius correction
        uint32_t k1[U], k2[U], rq[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t lid = seg_lid(sg, iu[u]);
            k1[u] = sg_philox_k23(c0b + 1u, lid, sg.key);
            k2[u] = sg_philox_k23(c0b + 1u + kNormalSalt2, lid, sg.key);
            rq[u] = a.bm_rq ? __ldg(a.bm_rq + k1[u]) : 0u;
        }
        if (W != 8 || !a.nb8) { // any width, or no neighbour table: one agent at a time
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const float x = opinion_mean<0>(a, sg, xin, iu[u], sg.width);
                if (vu[u]) xout[iu[u]] = opinion_noise(a, sg, trig, x, rq[u], k1[u], k2[u]);
            }
            continue;
        }
        // 2. weights (read once per tick: evict-first loads keep L2 for the
        //    opinions, which neighbours re-read), own opinions, and the first 8
        //    neighbours from the group-major table (each load instruction of a
        //    warp is one 128-byte line)
        int32_t m[U], nb[U][8];
        float wv[U][8], xo[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float4 *w4 = reinterpret_cast<const float4 *>(sg.weights + (int64_t)iu[u] * 8);
            const float4 w0 = __ldcs(w4), w1 = __ldcs(w4 + 1);
            wv[u][0] = w0.x, wv[u][1] = w0.y, wv[u][2] = w0.z, wv[u][3] = w0.w;
            wv[u][4] = w1.x, wv[u][5] = w1.y, wv[u][6] = w1.z, wv[u][7] = w1.w;
            xo[u] = xin[iu[u]];
#pragma unroll
            for (int j = 0; j < 8; ++j) nb[u][j] = __ldcs(a.nb8 + SG_NB8_AT(iu[u], j));
        }
        // 3. the row length is the count of valid entries (they come first)
#pragma unroll
        for (int u = 0; u < U; ++u) {
            m[u] = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                m[u] += nb[u][j] >= 0;
                if (nb[u][j] < 0) nb[u][j] = iu[u];
            }
        }
        // 4. neighbour opinions
        float xv[U][8];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < 8; ++j) xv[u][j] = __ldg(xin + nb[u][j]);
        // 5. weighted mean in row order (every multiply and add rounded), noise, store
#pragma unroll
        for (int u = 0; u < U; ++u) {
            float acc = 0.0f, norm = 0.0f;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (j < m[u]) {
                    acc = __fadd_rn(acc, __fmul_rn(wv[u][j], xv[u][j]));
                    norm = __fadd_rn(norm, fabsf(wv[u][j]));
                }
            const float x = norm > 0.0f ? __fdiv_rn(acc, norm) : xo[u];
            if (vu[u]) xout[iu[u]] = opinion_noise(a, sg, trig, x, rq[u], k1[u], k2[u]);
        }
    }
}

__global__ void offset_csr_kernel(int32_t *__restrict__ off, int64_t n1, int32_t edge_base,
                                  int32_t *__restrict__ idx, int64_t nnz, int32_t agent_base)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n1; i += stride) off[i] += edge_base;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += stride) idx[k] += agent_base;
}

// flag = 1 when offsets decrease, 2 when an index is outside [0, n) (either
// may win when both occur).
__global__ void check_csr_kernel(const int32_t *__restrict__ off, int64_t n, const int32_t *__restrict__ idx,
                                 int64_t nnz, int32_t *flag)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
        if (off[i + 1] < off[i]) *flag = 1;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += stride) {
        const int32_t v = idx[k];
        if (v < 0 || (int64_t)v >= n) *flag = 2;
    }
}

__global__ void copy_words_kernel(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst,
                                  int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__global__ void degree_count_kernel(const int32_t *__restrict__ idx, int64_t nnz,
                                    int32_t *__restrict__ cnt)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + idx[k], 1);
}

__global__ void transpose_fill_kernel(const int32_t *__restrict__ off,
                                      const int32_t *__restrict__ idx, int64_t n,
                                      int32_t *__restrict__ cursor, int32_t *__restrict__ tidx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        for (int32_t k = off[i]; k < off[i + 1]; ++k) {
            const int32_t d = idx[k];
            tidx[atomicAdd(cursor + d, 1)] = (int32_t)i;
        }
    }
}

} // namespace

cudaError_t sg_launch_sir_pull(const SgTickArgs &a, int variant, bool stats, int grid,
                               cudaStream_t st)
{
    if (variant == 1) {
        if (stats)
            sir_pull_kernel<1, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        else
            sir_pull_kernel<1, false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    } else {
        if (stats)
            sir_pull_kernel<2, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        else
            sir_pull_kernel<2, false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    }
    return cudaGetLastError();
}

// SM count of the current device: grids of the grid-stride kernels below are
// sized as a multiple of it.
static int current_sm_count()
{
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
        v = 1; // the launch that follows reports the device's error
    return v;
}

// Blocks of 256 threads for `work` items, at most 16 per SM (grid-stride loops).
static int stride_grid(int64_t work)
{
    const int64_t cap = (int64_t)current_sm_count() * 16;
    const int64_t b = (work + 255) / 256;
    return (int)(b < 1 ? 1 : b > cap ? cap : b);
}

cudaError_t sg_launch_opinion_tables(float2 *radius, uint32_t *rq, float2 *trig, cudaStream_t st)
{
    opinion_tables_kernel<<<current_sm_count() * 8, 256, 0, st>>>(radius, rq, trig);
    return cudaGetLastError();
}

cudaError_t sg_launch_opinion_noise_check(const SgTickArgs &a, const float *x, const uint32_t *k1, const uint32_t *k2,
                                          int64_t n, float *out, float *exact, uint8_t *slow, cudaStream_t st)
{
    opinion_noise_check_kernel<<<stride_grid(n), 256, 0, st>>>(a, x, k1, k2, n, out, exact, slow);
    return cudaGetLastError();
}

cudaError_t sg_launch_opinion_neighbours8(const int32_t *offsets, const int32_t *indices, int64_t n, int32_t *nb8,
                                          cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    opinion_neighbours8_kernel<<<stride_grid(n), 256, 0, st>>>(offsets, indices, n, nb8);
    return cudaGetLastError();
}

cudaError_t sg_launch_opinion_cos_check(const float2 *trig, int32_t k0, int32_t n, double *out, cudaStream_t st)
{
    opinion_cos_check_kernel<<<current_sm_count() * 8, 256, 0, st>>>(trig, k0, n, out);
    return cudaGetLastError();
}

// width: the weights per agent of every segment of the launch (8 takes the
// vector-load path). The grid is three persistent blocks per SM (the `grid`
// argument caps it).
cudaError_t sg_launch_opinion(const SgTickArgs &a, int grid, cudaStream_t st, int width)
{
    void (*k)(SgTickArgs) = width == 8 ? opinion_kernel<8> : opinion_kernel<0>;
    const size_t smem = a.bm_trig ? (size_t)SG_BM_TRIG_ENTRIES * sizeof(float2) : 0;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(opinion_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(SG_BM_TRIG_ENTRIES * sizeof(float2)));
        cudaFuncSetAttribute(opinion_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(SG_BM_TRIG_ENTRIES * sizeof(float2)));
    });
    const int per_thread = width == 8 ? 2 : 1;
    const int64_t nchunks = (int64_t)a.ntiles * (SG_TILE / (kOpinionThreads * per_thread));
    int64_t g = (int64_t)current_sm_count() * (width == 8 ? 2 : 3); // resident blocks per SM
    if (g > nchunks) g = nchunks;
    if (grid > 0 && g > (int64_t)grid * 4) g = (int64_t)grid * 4;
    if (g < 1) g = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)g);
    cfg.blockDim = dim3(kOpinionThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at{};
    if (a.l2_win) {
        at.id = cudaLaunchAttributeAccessPolicyWindow;
        at.val.accessPolicyWindow.base_ptr = const_cast<void *>(a.l2_win);
        at.val.accessPolicyWindow.num_bytes = a.l2_win_bytes;
        at.val.accessPolicyWindow.hitRatio = a.l2_win_hit;
        at.val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        at.val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = &at;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, k, a);
}

cudaError_t sg_launch_offset_csr(int32_t *off, int64_t n1, int32_t edge_base, int32_t *idx, int64_t nnz,
                                 int32_t agent_base, cudaStream_t st)
{
    const int64_t work = n1 > nnz ? n1 : nnz;
    if (work <= 0) return cudaSuccess;
    const int blocks = stride_grid(work);
    offset_csr_kernel<<<(int)blocks, 256, 0, st>>>(off, n1, edge_base, idx, nnz, agent_base);
    return cudaGetLastError();
}

cudaError_t sg_launch_check_csr(const int32_t *off, int64_t n, const int32_t *idx, int64_t nnz, int32_t *flag,
                                cudaStream_t st)
{
    const int64_t work = n > nnz ? n : nnz;
    if (work <= 0) return cudaSuccess;
    const int blocks = stride_grid(work);
    check_csr_kernel<<<(int)blocks, 256, 0, st>>>(off, n, idx, nnz, flag);
    return cudaGetLastError();
}

cudaError_t sg_launch_copy_words(const uint32_t *src, uint32_t *dst, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int blocks = stride_grid(n);
    copy_words_kernel<<<(int)blocks, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

size_t sg_transpose_scan_bytes(int64_t n)
{
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, (int32_t *)nullptr, (int32_t *)nullptr,
                                  (int)(n + 1));
    return bytes;
}

cudaError_t sg_transpose_csr(const int32_t *off, const int32_t *idx, int64_t n, int64_t nnz,
                             int32_t *toff, int32_t *tidx, int32_t *tmp, void *scan_tmp,
                             size_t scan_tmp_bytes, cudaStream_t st)
{
    cudaError_t err = cudaMemsetAsync(tmp, 0, (size_t)(n + 1) * sizeof(int32_t), st);
    if (err != cudaSuccess) return err;
    if (nnz > 0) {
        const int blocks = stride_grid(nnz);
        degree_count_kernel<<<(int)blocks, 256, 0, st>>>(idx, nnz, tmp);
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    size_t bytes = scan_tmp_bytes;
    err = cub::DeviceScan::ExclusiveSum(scan_tmp, bytes, tmp, toff, (int)(n + 1), st);
    if (err != cudaSuccess) return err;
    // cursor = copy of toff[0..n)
    err = cudaMemcpyAsync(tmp, toff, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    if (err != cudaSuccess) return err;
    if (n > 0) {
        const int blocks = stride_grid(n);
        transpose_fill_kernel<<<(int)blocks, 256, 0, st>>>(off, idx, n, tmp, tidx);
        err = cudaGetLastError();
    }
    return err;
}

cudaError_t sg_launch_frontier_build(const SgTickArgs &a, bool stats, int grid, cudaStream_t st)
{
    if (stats)
        frontier_build_kernel<true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    else
        frontier_build_kernel<false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sg_launch_frontier_step(const SgTickArgs &a, int variant, bool stats, int grid, cudaStream_t st)
{
    if (variant == 1) {
        if (stats)
            frontier_step_kernel<1, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        else
            frontier_step_kernel<1, false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    } else {
        if (stats)
            frontier_step_kernel<2, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        else
            frontier_step_kernel<2, false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t sg_launch_frontier_scatter(const SgTickArgs &a, int grid, cudaStream_t st)
{
    frontier_scatter_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}
