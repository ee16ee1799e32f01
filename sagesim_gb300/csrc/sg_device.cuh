// sg_device.cuh -- device helpers shared by the tick kernels' translation units
// (warp reductions, the neighbour scans of the three row-length bins, the
// SIR-B draw loops). Everything here is inline and has internal linkage.
#pragma once
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

} // namespace
