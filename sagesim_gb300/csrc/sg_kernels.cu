// sg_kernels.cu -- tick kernels for sm_103a.
//
// The tick semantics follow SAGESim's generated fused kernel
// (sagesim/model.py:2306-2408): every step reads tick-start values and writes a
// separate buffer; the next tick reads what this tick wrote. Here the two
// buffers ping-pong (buffer (par0 + r) & 1 is read at relative tick r), so the
// reference's per-tick write-back copy (model.py:2374-2389) disappears.
//
// Work decomposition: a persistent grid walks a tile list (tiles never straddle
// segments). Inside a tile, one thread takes one agent; an agent whose CSR row
// is longer than hub_deg is pushed to a shared-memory queue and processed by a
// whole warp after the thread pass (ballot/popc over 32 neighbours per step).
// That is the degree binning: short rows stay thread-per-agent with no
// divergence from hubs, hub rows are read coalesced by a warp.
#include <cub/device/device_scan.cuh>

#include "sg_kernels.h"
#include "sg_philox.h"

#define FULL_MASK 0xffffffffu

namespace {

constexpr int kWarps = SG_SIR_THREADS / 32;
constexpr uint32_t kNormalSalt2 = 73856093u; // sagesim/math_utils.py:252

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

// Block-reduces four counters and adds them to dst[0..3] (one atomic each).
__device__ __forceinline__ void block_flush4(unsigned long long v0, unsigned long long v1,
                                             unsigned long long v2, unsigned long long v3,
                                             unsigned long long *dst,
                                             unsigned long long (*sh)[kWarps])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v0 = warp_sum(v0);
    v1 = warp_sum(v1);
    v2 = warp_sum(v2);
    v3 = warp_sum(v3);
    if (lane == 0) {
        sh[0][warp] = v0;
        sh[1][warp] = v1;
        sh[2][warp] = v2;
        sh[3][warp] = v3;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            unsigned long long x = lane < kWarps ? sh[k][lane] : 0ull;
            x = warp_sum(x);
            if (lane == 0 && x) atomicAdd(dst + k, x);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ uint32_t seg_lid(const SgSeg &sg, int32_t i)
{
    return sg.lids ? __ldg(sg.lids + i) : (uint32_t)(i - sg.lid_base);
}

// ---- neighbour scans ------------------------------------------------------------
// Every scan is counted, never ordered: SIR-A needs "any infected neighbour",
// SIR-B needs only how many of the scanned neighbours are infected (the j-th
// infected one draws salt 2 + j whichever neighbour it is). So rows are read
// in batches whose loads are all independent (memory-level parallelism), and
// the draws for a batch's c infected neighbours are tested together.
//
// Three bins by row length, all warp-synchronous: a lane scans its own row
// when it has <= kThreadRow entries (4 independent gathers per step); the
// whole warp scans rows of <= kWarpRow entries (128 per step); rows longer
// than that ("mega" rows, a few dozen in a 10^7-agent power-law graph) are
// listed at setup and scanned by dedicated blocks (1024 entries per step).
constexpr int kBatch = 4;
constexpr int32_t kThreadRow = 32; // default of SgTickArgs::thread_row

__device__ __forceinline__ int32_t thread_row_of(const SgTickArgs &a)
{
    return a.thread_row > 0 ? a.thread_row : kThreadRow;
}

// Number of infected entries among row[k .. min(k+4, e)), e > k.
__device__ __forceinline__ int batch_count(const int32_t *__restrict__ idx,
                                           const int32_t *__restrict__ sin, int32_t k, int32_t e,
                                           int32_t ci)
{
    const int32_t last = e - 1;
    const int32_t n0 = __ldg(idx + k);
    const int32_t n1 = __ldg(idx + min(k + 1, last));
    const int32_t n2 = __ldg(idx + min(k + 2, last));
    const int32_t n3 = __ldg(idx + min(k + 3, last));
    const int32_t s0 = __ldg(sin + n0), s1 = __ldg(sin + n1), s2 = __ldg(sin + n2),
                  s3 = __ldg(sin + n3);
    return (s0 == ci) + (k + 1 < e && s1 == ci) + (k + 2 < e && s2 == ci) + (k + 3 < e && s3 == ci);
}

// SIR-B outcome for one agent from its row, lane path.
__device__ __forceinline__ bool trials_thread(const int32_t *__restrict__ idx,
                                              const int32_t *__restrict__ sin, int32_t b,
                                              int32_t e, int32_t ci, uint32_t c0b, uint32_t lid,
                                              uint32_t key, uint32_t kinf)
{
    uint32_t j = 0;
    for (int32_t k = b; k < e; k += kBatch) {
        const int c = batch_count(idx, sin, k, e, ci);
        for (int q = 0; q < c; ++q, ++j)
            if (sg_philox_k23(c0b + 2u + j, lid, key) < kinf) return true;
    }
    return false;
}

__device__ __forceinline__ bool any_infected_thread(const int32_t *__restrict__ idx,
                                                    const int32_t *__restrict__ sin, int32_t b,
                                                    int32_t e, int32_t ci)
{
    for (int32_t k = b; k < e; k += kBatch)
        if (batch_count(idx, sin, k, e, ci)) return true;
    return false;
}

__device__ __forceinline__ int32_t count_thread(const int32_t *__restrict__ idx,
                                                const int32_t *__restrict__ sin, int32_t b,
                                                int32_t e, int32_t ci)
{
    int32_t c = 0;
    for (int32_t k = b; k < e; k += kBatch) c += batch_count(idx, sin, k, e, ci);
    return c;
}

// Warp path: each lane takes 4 entries per step (128 per warp step).
__device__ __forceinline__ int warp_batch_count(const int32_t *__restrict__ idx,
                                                const int32_t *__restrict__ sin, int32_t k0,
                                                int32_t e, int32_t ci, int lane)
{
    const int32_t k = k0 + lane;
    const bool v0 = k < e, v1 = k + 32 < e, v2 = k + 64 < e, v3 = k + 96 < e;
    const int32_t last = e - 1;
    const int32_t n0 = __ldg(idx + min(k, last));
    const int32_t n1 = __ldg(idx + min(k + 32, last));
    const int32_t n2 = __ldg(idx + min(k + 64, last));
    const int32_t n3 = __ldg(idx + min(k + 96, last));
    const int32_t s0 = __ldg(sin + n0), s1 = __ldg(sin + n1), s2 = __ldg(sin + n2),
                  s3 = __ldg(sin + n3);
    int c = (v0 && s0 == ci) + (v1 && s1 == ci) + (v2 && s2 == ci) + (v3 && s3 == ci);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(FULL_MASK, c, o);
    return c;
}

// Tests draws j0 .. j0+c-1 (salt 2 + j) across the warp; true if any is below beta.
__device__ __forceinline__ bool warp_draws(uint32_t j0, int c, uint32_t c0b, uint32_t lid,
                                           uint32_t key, uint32_t kinf, int lane)
{
    for (int q0 = 0; q0 < c; q0 += 32) {
        const bool ok = (q0 + lane < c) &&
                        (sg_philox_k23(c0b + 2u + j0 + (uint32_t)(q0 + lane), lid, key) < kinf);
        if (__any_sync(FULL_MASK, ok)) return true;
    }
    return false;
}

// SIR-B outcome for every lane's agent given its infected-neighbour count k
// (act = the lane has a susceptible agent with k > 0). Each lane tests its
// first kLaneDraws draws itself; agents that need more share the warp, which
// tests 32 draws (salt 2 + j) per step. Every lane of the warp must call it.
constexpr int32_t kLaneDraws = 2;

__device__ __forceinline__ bool sirb_infected(bool act, int32_t k, uint32_t c0b, uint32_t lid,
                                              uint32_t key, uint32_t kinf, int lane)
{
    bool inf = false;
    int32_t done = 0;
    if (act) {
        done = k < kLaneDraws ? k : kLaneDraws;
        for (int32_t j = 0; j < done; ++j)
            if (sg_philox_k23(c0b + 2u + (uint32_t)j, lid, key) < kinf) {
                inf = true;
                break;
            }
    }
    unsigned m = __ballot_sync(FULL_MASK, act && !inf && k > done);
    while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const int32_t bk = __shfl_sync(FULL_MASK, k, l);
        const uint32_t bc = __shfl_sync(FULL_MASK, c0b, l);
        const uint32_t bl = __shfl_sync(FULL_MASK, lid, l);
        const uint32_t bkey = __shfl_sync(FULL_MASK, key, l);
        const uint32_t bkinf = __shfl_sync(FULL_MASK, kinf, l);
        const bool hit = warp_draws((uint32_t)kLaneDraws, bk - kLaneDraws, bc, bl, bkey, bkinf, lane);
        if (lane == l) inf = hit;
    }
    return inf;
}

// VARIANT 1: any infected; 2: SIR-B trials; 0: count (returned through *count).
template <int VARIANT>
__device__ __forceinline__ bool warp_row(const int32_t *__restrict__ idx,
                                         const int32_t *__restrict__ sin, int32_t b, int32_t e,
                                         int32_t ci, uint32_t c0b, uint32_t lid, uint32_t key,
                                         uint32_t kinf, int lane, int32_t *count)
{
    uint32_t j = 0;
    for (int32_t k0 = b; k0 < e; k0 += 128) {
        const int c = warp_batch_count(idx, sin, k0, e, ci, lane);
        if (VARIANT == 1 && c) return true;
        if (VARIANT == 2 && c) {
            if (warp_draws(j, c, c0b, lid, key, kinf, lane)) return true;
        }
        j += (uint32_t)c;
    }
    if (count) *count = (int32_t)j;
    return false;
}

// Block path for mega rows: 256 threads x 4 entries per step; the result is
// broadcast through __syncthreads_or / a shared counter. Called by every
// thread of the block.
template <int VARIANT>
__device__ __forceinline__ bool block_row(const int32_t *__restrict__ idx,
                                          const int32_t *__restrict__ sin, int32_t b, int32_t e,
                                          int32_t ci, uint32_t c0b, uint32_t lid, uint32_t key,
                                          uint32_t kinf, int32_t *sh_count, int32_t *count)
{
    const int tid = threadIdx.x;
    __syncthreads(); // previous users of *sh_count are done
    if (tid == 0) *sh_count = 0;
    __syncthreads();
    for (int32_t k0 = b; k0 < e; k0 += 4 * SG_SIR_THREADS) {
        const int32_t k = k0 + tid;
        const int32_t last = e - 1;
        const int32_t n0 = __ldg(idx + min(k, last));
        const int32_t n1 = __ldg(idx + min(k + SG_SIR_THREADS, last));
        const int32_t n2 = __ldg(idx + min(k + 2 * SG_SIR_THREADS, last));
        const int32_t n3 = __ldg(idx + min(k + 3 * SG_SIR_THREADS, last));
        const int mine = (k < e && __ldg(sin + n0) == ci) +
                         (k + SG_SIR_THREADS < e && __ldg(sin + n1) == ci) +
                         (k + 2 * SG_SIR_THREADS < e && __ldg(sin + n2) == ci) +
                         (k + 3 * SG_SIR_THREADS < e && __ldg(sin + n3) == ci);
        if (mine) atomicAdd(sh_count, mine);
        if (VARIANT == 1) {
            if (__syncthreads_or(mine != 0)) return true;
        }
    }
    __syncthreads();
    const int32_t total = *sh_count;
    if (count) *count = total;
    if (VARIANT == 2) {
        bool ok = false;
        for (int32_t q = tid; q < total && !ok; q += SG_SIR_THREADS)
            ok = sg_philox_k23(c0b + 2u + (uint32_t)q, lid, key) < kinf;
        return __syncthreads_or(ok) != 0;
    }
    return false;
}

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

// ---- count strategy -------------------------------------------------------------
// cnt[i] = number of infected agents in row i, kept for susceptible agents
// (the only ones that read it; agents never return to S). A susceptible agent
// then needs only cnt[i]: SIR-A infects iff cnt > 0 and u < beta, SIR-B iff
// one of the draws salt 2 .. 2+cnt-1 is below beta. Agents whose infected
// status changed are appended to their tile's slice of the change list
// (tile t owns changes[tile.begin ..] and tile_nch[t]; no global atomics);
// the scatter kernel then adds +-1 to cnt along their transpose rows.

__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_init_kernel(SgTickArgs a)
{
    __shared__ int32_t sh_count;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile_blocks = (int)gridDim.x - a.mega_blocks;
    if ((int)blockIdx.x >= tile_blocks) {
        for (int q = (int)blockIdx.x - tile_blocks; q < a.nmega; q += a.mega_blocks) {
            const SgMega mg = a.mega[q];
            const SgSeg &sg = a.segs[mg.seg];
            const int32_t *__restrict__ sin = (const int32_t *)((sg.par0 & 1) ? a.buf1 : a.buf0);
            const int32_t h = mg.agent;
            if (sin[h] != sg.cs) continue;
            int32_t c = 0;
            block_row<0>(a.idx, sin, a.off[h], a.off[h + 1], sg.ci, 0, 0, 0, 0, &sh_count, &c);
            if (tid == 0) a.cnt[h] = c;
        }
        return;
    }
    for (int t = blockIdx.x; t < a.ntiles; t += tile_blocks) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int32_t *__restrict__ sin = (const int32_t *)((sg.par0 & 1) ? a.buf1 : a.buf0);
        const int32_t ci = sg.ci, cs = sg.cs;
        for (int32_t wbase = tile.begin + warp * 32; wbase < tile.end; wbase += SG_SIR_THREADS) {
            const int32_t i = wbase + lane;
            bool medium = false;
            int32_t b = 0, e = 0;
            if (i < tile.end && sin[i] == cs) {
                b = a.off[i];
                e = a.off[i + 1];
                if (e - b > a.mega_row) {
                    // mega block
                } else if (e - b > thread_row_of(a)) {
                    medium = true;
                } else {
                    a.cnt[i] = count_thread(a.idx, sin, b, e, ci);
                }
            }
            unsigned m = __ballot_sync(FULL_MASK, medium);
            while (m) {
                const int l = __ffs(m) - 1;
                m &= m - 1;
                const int32_t hb = __shfl_sync(FULL_MASK, b, l);
                const int32_t he = __shfl_sync(FULL_MASK, e, l);
                int32_t c = 0;
                warp_row<0>(a.idx, sin, hb, he, ci, 0, 0, 0, 0, lane, &c);
                if (lane == l) a.cnt[i] = c;
            }
        }
    }
}

constexpr int kPerThread = SG_TILE / SG_SIR_THREADS; // agents per thread in a tile

// Warp-dense SIR-B draws. Lane l holds up to kCountPer susceptible agents; agent
// q needs draws j = 0 .. k[q]-1 (salt 2 + j) until one is below beta. The warp
// lays out the first min(k, kWarpDenseCap) draws of all its agents in one
// sequence (exclusive scan of the lanes' totals) and evaluates 32 of them per
// step, one per lane: the owner of draw d is found by a shuffle binary search
// over the lanes' scan values. Hits are flagged in shared memory. Agents with
// more draws and no hit continue with 32-wide warp batches. Returns the bit
// mask of the calling lane's infected agents. Every lane must call it.
constexpr int32_t kWarpDenseCap = 32;

template <int P>
__device__ __forceinline__ unsigned warp_dense_sirb(const int32_t (&k)[P], const uint32_t (&lid)[P],
                                                    uint32_t c0b, uint32_t key, uint32_t kinf, int lane,
                                                    unsigned char *flags /* 32 * P bytes of this warp */)
{
    int32_t c[P], tot = 0;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        c[q] = k[q] < kWarpDenseCap ? k[q] : kWarpDenseCap;
        tot += c[q];
        flags[lane * P + q] = 0;
    }
    int32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    const int32_t base = x - tot;
    const int32_t W = __shfl_sync(FULL_MASK, x, 31);
    __syncwarp();
    for (int32_t d0 = 0; d0 < W; d0 += 32) {
        const int32_t d = d0 + lane;
        int32_t lo = 0; // owner: the last lane with base <= d
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int32_t b = __shfl_sync(FULL_MASK, base, (lo + step) & 31);
            if (lo + step < 32 && b <= d) lo += step;
        }
        int32_t off = d - __shfl_sync(FULL_MASK, base, lo);
        int32_t qsel = 0;
        uint32_t l = 0;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int32_t cq = __shfl_sync(FULL_MASK, c[q], lo);
            const uint32_t lq = __shfl_sync(FULL_MASK, lid[q], lo);
            if (qsel == q) {
                if (off < cq) {
                    l = lq;
                    qsel = q + 100; // found: stop advancing
                } else {
                    off -= cq;
                    qsel = q + 1;
                }
            }
        }
        if (d < W && qsel >= 100 && sg_philox_k23(c0b + 2u + (uint32_t)off, l, key) < kinf)
            flags[lo * P + (qsel - 100)] = 1;
    }
    __syncwarp();
    unsigned bits = 0;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        bool inf = flags[lane * P + q] != 0;
        unsigned m = __ballot_sync(FULL_MASK, !inf && k[q] > kWarpDenseCap);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const int32_t bk = __shfl_sync(FULL_MASK, k[q], src);
            const uint32_t bl = __shfl_sync(FULL_MASK, lid[q], src);
            const bool h = warp_draws((uint32_t)kWarpDenseCap, bk - kWarpDenseCap, c0b, bl, key, kinf, lane);
            if (lane == src) inf = h;
        }
        if (inf) bits |= 1u << q;
    }
    __syncwarp(); // flags are reused by the next call
    return bits;
}

// A changed agent whose transpose row is longer than kSegRow is handed to the
// scatter as row segments of kSegRow entries on their own work list, so no
// single warp walks a hub's whole row; the chunk pass skips such rows.
constexpr int32_t kSegRow = 256;

__device__ __forceinline__ void publish_long_row(const SgTickArgs &a, int32_t g, int32_t delta)
{
    const int32_t b = __ldg(a.toff + g), e = __ldg(a.toff + g + 1);
    if (e - b <= kSegRow) return;
    const int32_t nseg = (e - b + kSegRow - 1) / kSegRow;
    const int32_t base = atomicAdd(a.nrowsegs + a.r, nseg);
    for (int32_t j = 0; j < nseg; ++j) {
        const int32_t sb = b + j * kSegRow;
        a.rowsegs[base + j] = SgRowSeg{sb, min(sb + kSegRow, e), delta, 0};
    }
}

// Count-strategy step. Late in an epidemic this is a streaming pass over every
// agent; at its peak most susceptible agents draw. Flavours (all give the
// same result; the autotuner picks one):
//   PER    4: one agent per thread per 256-agent stripe (scalar loads); 8: two
//          runs of 4 consecutive agents per thread read with 128-bit loads
//   DENSE  SIR-B draws laid out warp-densely (warp_dense_sirb) instead of per-lane loops
//   LAZY   the count and RNG key are loaded only for agents that need them (a
//          second round trip) instead of unconditionally with the state
// The segment's parameters stay in registers while consecutive tiles share a
// segment, and changes go to the tile's own slice of the change list.
template <int VARIANT, bool STATS, bool INPLACE, int PER, bool DENSE, bool LAZY>
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_step_kernel(SgTickArgs a)
{
    static_assert(SG_TILE % (SG_SIR_THREADS * PER) == 0, "tile must be whole passes");
    __shared__ unsigned long long red[4][kWarps];
    __shared__ int32_t nch, chunk_base;
    __shared__ unsigned char wflags[DENSE ? SG_SIR_THREADS * PER : 1];
    const int tid = threadIdx.x, lane = tid & 31;
    int32_t cur_seg = -1;
    int64_t tick = 0, end_tick = 0;
    uint32_t c0b = 0, key = 0, kinf = 0, krec = 0;
    int32_t cs = 0, ci = 0, cr = 0, par = 0, lid_base = 0;
    const uint32_t *lids = nullptr;
    SgPhiloxKeys ks = sg_philox_keys(0);
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        if (tile.seg != cur_seg) {
            const SgSeg &sg = a.segs[tile.seg];
            cur_seg = tile.seg;
            tick = sg.tick0 + a.r;
            end_tick = sg.end_tick;
            c0b = sg_c0base(tick);
            key = sg.key;
            ks = sg_philox_keys(key);
            kinf = sg.kinf;
            krec = sg.krec;
            cs = sg.cs;
            ci = sg.ci;
            cr = sg.cr;
            par = INPLACE ? 0 : ((sg.par0 + a.r) & 1);
            lids = sg.lids;
            lid_base = sg.lid_base;
        }
        if (tick >= end_tick) {
            if (tid == 0) a.tile_nch[t] = 0;
            continue;
        }
        const int32_t *sin = (const int32_t *)(par ? a.buf1 : a.buf0);
        int32_t *sout = (int32_t *)(INPLACE ? a.buf0 : (par ? a.buf0 : a.buf1));
        int32_t *tchanges = a.changes + tile.begin;
        unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;
        if (tid == 0) nch = 0;
        __syncthreads();
        for (int32_t pass = tile.begin; pass < tile.end; pass += SG_SIR_THREADS * PER) {
            // agent of slot q: PER == 4 -> strided (pass + q*256 + tid, scalar
            // coalesced loads); PER == 8 -> two runs of 4 consecutive agents per
            // thread (pass + (q/4)*1024 + tid*4 + q%4) read with 128-bit loads
            auto agent = [&](int q) -> int32_t {
                return PER == 8 ? pass + (q >> 2) * (SG_SIR_THREADS * 4) + tid * 4 + (q & 3)
                                : pass + q * SG_SIR_THREADS + tid;
            };
            int32_t s[PER], k[PER];
            uint32_t lid[PER];
            if (PER == 8) {
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    const int32_t b = agent(g * 4);
                    if (b + 3 < tile.end && (b & 3) == 0) {
                        const int4 v = *reinterpret_cast<const int4 *>(sin + b);
                        s[g * 4] = v.x;
                        s[g * 4 + 1] = v.y;
                        s[g * 4 + 2] = v.z;
                        s[g * 4 + 3] = v.w;
                        if (!LAZY) {
                            const int4 c = *reinterpret_cast<const int4 *>(a.cnt + b);
                            k[g * 4] = c.x;
                            k[g * 4 + 1] = c.y;
                            k[g * 4 + 2] = c.z;
                            k[g * 4 + 3] = c.w;
                            if (lids) {
                                const uint4 l = __ldg(reinterpret_cast<const uint4 *>(lids + b));
                                lid[g * 4] = l.x;
                                lid[g * 4 + 1] = l.y;
                                lid[g * 4 + 2] = l.z;
                                lid[g * 4 + 3] = l.w;
                            } else {
#pragma unroll
                                for (int e = 0; e < 4; ++e) lid[g * 4 + e] = (uint32_t)(b + e - lid_base);
                            }
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int32_t i = b + e;
                            const bool v = i < tile.end;
                            s[g * 4 + e] = v ? sin[i] : INT32_MIN;
                            if (!LAZY) {
                                k[g * 4 + e] = v ? a.cnt[i] : 0;
                                lid[g * 4 + e] = lids ? (v ? __ldg(lids + i) : 0u) : (uint32_t)(i - lid_base);
                            }
                        }
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int32_t i = agent(q);
                    const bool v = i < tile.end;
                    s[q] = v ? sin[i] : INT32_MIN;
                    if (!LAZY) {
                        k[q] = v ? a.cnt[i] : 0;
                        lid[q] = lids ? (v ? __ldg(lids + i) : 0u) : (uint32_t)(i - lid_base);
                    }
                }
            }
            if (LAZY) {
#pragma unroll
                for (int q = 0; q < PER; ++q) k[q] = s[q] == cs ? a.cnt[agent(q)] : 0;
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int32_t i = agent(q);
                    lid[q] = (s[q] == ci || (s[q] == cs && k[q] > 0))
                                 ? (lids ? __ldg(lids + i) : (uint32_t)(i - lid_base))
                                 : 0u;
                }
            }
            unsigned inf_bits = 0;
            if (VARIANT == 2 && DENSE) {
                int32_t kd[PER];
#pragma unroll
                for (int q = 0; q < PER; ++q) kd[q] = s[q] == cs ? k[q] : 0;
                inf_bits = warp_dense_sirb<PER>(kd, lid, c0b, key, kinf, lane, wflags + (tid >> 5) * 32 * PER);
            }
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int32_t i = agent(q);
                int32_t out = s[q];
                bool has = false;
                int32_t code = 0;
                if (s[q] == ci) {
                    if (sg_philox_k23_keys(c0b + 1u, lid[q], ks) < krec) {
                        out = cr;
                        has = true;
                        code = ~i;
                    }
                } else if (s[q] == cs && k[q] > 0) {
                    bool inf = false;
                    if (VARIANT == 1) {
                        inf = sg_philox_k23_keys(c0b + 1u, lid[q], ks) < kinf;
                    } else if (DENSE) {
                        inf = ((inf_bits >> q) & 1u) != 0;
                    } else {
                        for (int32_t j = 0; j < k[q]; ++j)
                            if (sg_philox_k23_keys(c0b + 2u + (uint32_t)j, lid[q], ks) < kinf) {
                                inf = true;
                                break;
                            }
                    }
                    if (inf) {
                        out = ci;
                        has = true;
                        code = i;
                    }
                }
                if (i < tile.end) {
                    if (!INPLACE || has) sout[i] = out;
                    if (STATS) {
                        if (s[q] == cs) eS += (unsigned long long)(__ldg(a.off + i + 1) - __ldg(a.off + i));
                        nS += (out == cs);
                        nI += (out == ci);
                        nR += (out == cr);
                    }
                }
                const unsigned m = __ballot_sync(FULL_MASK, has);
                if (m) {
                    const int leader = __ffs(m) - 1;
                    int32_t pos = 0;
                    if (lane == leader) pos = atomicAdd(&nch, __popc(m));
                    pos = __shfl_sync(FULL_MASK, pos, leader);
                    if (has) tchanges[pos + __popc(m & ((1u << lane) - 1u))] = code;
                }
                if (has && a.rowsegs) publish_long_row(a, i, code >= 0 ? 1 : -1);
            }
        }
        __syncthreads();
        {
            // publish the tile's change count and its 32-change chunks to the
            // scatter's work list (one atomic per tile with changes)
            const int32_t n = nch;
            const int32_t c = (n + 31) >> 5;
            if (tid == 0) {
                a.tile_nch[t] = n;
                if (a.chunks && n > 0) chunk_base = atomicAdd(a.nchunks + a.r, c);
            }
            __syncthreads();
            if (a.chunks && n > 0) {
                const int32_t base = chunk_base;
                for (int32_t j = tid; j < c; j += SG_SIR_THREADS) a.chunks[base + j] = SgChunk{t, j};
            }
        }
        if (STATS && a.segs[tile.seg].stats)
            block_flush4(nS, nI, nR, eS, a.segs[tile.seg].stats + 4 * (int64_t)a.r, red);
        __syncthreads(); // nch is reset by the next tile
    }
}

// Warp-synchronous: each warp takes 32 changes of a tile; short transpose rows
// are updated by their lane, longer ones by the whole warp.
// ±1 along the transpose rows of one warp's 32 changes of tile t (q0 = first).
__device__ __forceinline__ void scatter_changes(const SgTickArgs &a, const int32_t *tchanges, int32_t q0,
                                                int32_t n, int lane)
{
    const int32_t q = q0 + lane;
    const bool valid = q < n;
    const int32_t c = valid ? tchanges[q] : 0;
    const int32_t g = c >= 0 ? c : ~c;
    const int32_t delta = c >= 0 ? 1 : -1;
    int32_t b = 0, e = 0;
    if (valid) {
        b = __ldg(a.toff + g);
        e = __ldg(a.toff + g + 1);
    }
    if (a.rowsegs && e - b > kSegRow) e = b; // handled through the row-segment list
    const bool long_row = e - b > thread_row_of(a);
    if (!long_row) {
        for (int32_t k = b; k < e; k += 4) {
            const int32_t last = e - 1;
            const int32_t d0 = __ldg(a.tidx + k);
            const int32_t d1 = __ldg(a.tidx + min(k + 1, last));
            const int32_t d2 = __ldg(a.tidx + min(k + 2, last));
            const int32_t d3 = __ldg(a.tidx + min(k + 3, last));
            atomicAdd(a.cnt + d0, delta);
            if (k + 1 < e) atomicAdd(a.cnt + d1, delta);
            if (k + 2 < e) atomicAdd(a.cnt + d2, delta);
            if (k + 3 < e) atomicAdd(a.cnt + d3, delta);
        }
    }
    unsigned m = __ballot_sync(FULL_MASK, long_row);
    while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const int32_t hb = __shfl_sync(FULL_MASK, b, l);
        const int32_t he = __shfl_sync(FULL_MASK, e, l);
        const int32_t hd = __shfl_sync(FULL_MASK, delta, l);
        for (int32_t k = hb + lane; k < he; k += 32) atomicAdd(a.cnt + __ldg(a.tidx + k), hd);
    }
}

// Work-list form: warps take the tick's non-empty 32-change chunks, so a tile
// with thousands of changes is spread over many warps.
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_scatter_chunks_kernel(SgTickArgs a)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int32_t nck = a.nchunks[a.r];
    for (int32_t w = blockIdx.x * kWarps + warp; w < nck; w += gridDim.x * kWarps) {
        const SgChunk ck = a.chunks[w];
        scatter_changes(a, a.changes + a.tiles[ck.tile].begin, ck.chunk * 32, __ldg(a.tile_nch + ck.tile), lane);
    }
    if (a.rowsegs) {
        const int32_t nsg = a.nrowsegs[a.r];
        for (int32_t w = blockIdx.x * kWarps + warp; w < nsg; w += gridDim.x * kWarps) {
            const SgRowSeg sgm = a.rowsegs[w];
            for (int32_t k = sgm.begin + lane; k < sgm.end; k += 32) atomicAdd(a.cnt + __ldg(a.tidx + k), sgm.delta);
        }
    }
}

__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_scatter_kernel(SgTickArgs a)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const int32_t n = a.tile_nch[t];
        if (n == 0) continue;
        const int32_t *tchanges = a.changes + a.tiles[t].begin;
        for (int32_t q0 = warp * 32; q0 < n; q0 += SG_SIR_THREADS) {
            const int32_t q = q0 + lane;
            const bool valid = q < n;
            const int32_t c = valid ? tchanges[q] : 0;
            const int32_t g = c >= 0 ? c : ~c;
            const int32_t delta = c >= 0 ? 1 : -1;
            int32_t b = 0, e = 0;
            if (valid) {
                b = __ldg(a.toff + g);
                e = __ldg(a.toff + g + 1);
            }
            const bool long_row = e - b > thread_row_of(a);
            if (!long_row) {
                for (int32_t k = b; k < e; k += 4) {
                    const int32_t last = e - 1;
                    const int32_t d0 = __ldg(a.tidx + k);
                    const int32_t d1 = __ldg(a.tidx + min(k + 1, last));
                    const int32_t d2 = __ldg(a.tidx + min(k + 2, last));
                    const int32_t d3 = __ldg(a.tidx + min(k + 3, last));
                    atomicAdd(a.cnt + d0, delta);
                    if (k + 1 < e) atomicAdd(a.cnt + d1, delta);
                    if (k + 2 < e) atomicAdd(a.cnt + d2, delta);
                    if (k + 3 < e) atomicAdd(a.cnt + d3, delta);
                }
            }
            unsigned m = __ballot_sync(FULL_MASK, long_row);
            while (m) {
                const int l = __ffs(m) - 1;
                m &= m - 1;
                const int32_t hb = __shfl_sync(FULL_MASK, b, l);
                const int32_t he = __shfl_sync(FULL_MASK, e, l);
                const int32_t hd = __shfl_sync(FULL_MASK, delta, l);
                for (int32_t k = hb + lane; k < he; k += 32) atomicAdd(a.cnt + __ldg(a.tidx + k), hd);
            }
        }
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
// (sagesim/math_utils.py:231-255: u1 salt 1, u2 salt 1 + 73856093, +1e-10 guard).
__global__ void __launch_bounds__(SG_SIR_THREADS) opinion_kernel(SgTickArgs a)
{
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int64_t tick = sg.tick0 + a.r;
        if (tick >= sg.end_tick) continue;
        const int par = (sg.par0 + a.r) & 1;
        const float *__restrict__ xin = (const float *)(par ? a.buf1 : a.buf0);
        float *__restrict__ xout = (float *)(par ? a.buf0 : a.buf1);
        const uint32_t c0b = sg_c0base(tick);
        const int32_t width = sg.width;
        for (int32_t i = tile.begin + threadIdx.x; i < tile.end; i += SG_SIR_THREADS) {
            const int32_t b = __ldg(a.off + i);
            int32_t m = __ldg(a.off + i + 1) - b;
            if (m > width) m = width;
            const float *__restrict__ w = sg.weights + (int64_t)i * width;
            float acc = 0.0f, norm = 0.0f;
            for (int32_t j = 0; j < m; ++j) {
                const float wj = __ldg(w + j);
                const float xj = __ldg(xin + __ldg(a.idx + b + j));
                acc = __fadd_rn(acc, __fmul_rn(wj, xj));
                norm = __fadd_rn(norm, fabsf(wj));
            }
            float x = xin[i];
            if (norm > 0.0f) x = __fdiv_rn(acc, norm);
            const uint32_t lid = seg_lid(sg, i);
            const double u1 = (double)sg_philox_k23(c0b + 1u, lid, sg.key) / 8388608.0;
            const double u2 =
                (double)sg_philox_k23(c0b + 1u + kNormalSalt2, lid, sg.key) / 8388608.0;
            const double r = sqrt(__dmul_rn(-2.0, log(__dadd_rn(u1, 1e-10))));
            const double z = __dmul_rn(r, cos(__dmul_rn(6.283185307179586, u2)));
            double y = __dadd_rn((double)x, __dmul_rn(sg.sigma, z));
            if (y < 0.0) y = 0.0;
            if (y > 1.0) y = 1.0;
            xout[i] = (float)y;
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

cudaError_t sg_launch_sir_count_init(const SgTickArgs &a, int grid, cudaStream_t st)
{
    sir_count_init_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

template <int V, bool P>
static void count_step_flavour(const SgTickArgs &a, int flavour, int grid, cudaStream_t st)
{
    const bool per8 = flavour & SG_FLAVOUR_PER8, lazy = flavour & SG_FLAVOUR_LAZY;
    const bool dense = V == 2 && (flavour & SG_FLAVOUR_DENSE);
#define SG_CF(N, D, L) sir_count_step_kernel<V, false, P, N, D, L><<<grid, SG_SIR_THREADS, 0, st>>>(a)
    if (per8) {
        if (dense) {
            if (lazy) SG_CF(8, true, true); else SG_CF(8, true, false);
        } else {
            if (lazy) SG_CF(8, false, true); else SG_CF(8, false, false);
        }
    } else {
        if (dense) {
            if (lazy) SG_CF(4, true, true); else SG_CF(4, true, false);
        } else {
            if (lazy) SG_CF(4, false, true); else SG_CF(4, false, false);
        }
    }
#undef SG_CF
}

cudaError_t sg_launch_sir_count_step(const SgTickArgs &a, int variant, bool stats, bool inplace,
                                     int grid, cudaStream_t st)
{
    if (stats) { // statistics runs use one flavour
        if (variant == 1) {
            if (inplace) sir_count_step_kernel<1, true, true, 4, false, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
            else sir_count_step_kernel<1, true, false, 4, false, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        } else {
            if (inplace) sir_count_step_kernel<2, true, true, 4, true, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
            else sir_count_step_kernel<2, true, false, 4, true, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        }
        return cudaGetLastError();
    }
    if (variant == 1) {
        if (inplace) count_step_flavour<1, true>(a, a.flavour, grid, st);
        else count_step_flavour<1, false>(a, a.flavour, grid, st);
    } else {
        if (inplace) count_step_flavour<2, true>(a, a.flavour, grid, st);
        else count_step_flavour<2, false>(a, a.flavour, grid, st);
    }
    return cudaGetLastError();
}

cudaError_t sg_launch_sir_count_scatter(const SgTickArgs &a, int grid, cudaStream_t st)
{
    if (a.chunks)
        sir_count_scatter_chunks_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
    else
        sir_count_scatter_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sg_launch_opinion(const SgTickArgs &a, int grid, cudaStream_t st)
{
    opinion_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sg_launch_offset_csr(int32_t *off, int64_t n1, int32_t edge_base, int32_t *idx, int64_t nnz,
                                 int32_t agent_base, cudaStream_t st)
{
    const int64_t work = n1 > nnz ? n1 : nnz;
    if (work <= 0) return cudaSuccess;
    int64_t blocks = (work + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    offset_csr_kernel<<<(int)blocks, 256, 0, st>>>(off, n1, edge_base, idx, nnz, agent_base);
    return cudaGetLastError();
}

cudaError_t sg_launch_copy_words(const uint32_t *src, uint32_t *dst, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
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
        int64_t blocks = (nnz + 255) / 256;
        if (blocks > 152 * 16) blocks = 152 * 16;
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
        int64_t blocks = (n + 255) / 256;
        if (blocks > 152 * 16) blocks = 152 * 16;
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
