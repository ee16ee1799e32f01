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
    return sg.lids ? (uint32_t)(uint64_t)sg.lids[i] : (uint32_t)(i - sg.lid_base);
}

// ---- pull strategy ------------------------------------------------------------

// SIR-A (tests/test_simulation.py:24-43): infected iff u < beta and any
// neighbour is infected. u was drawn by the caller; this only scans.
__device__ __forceinline__ bool any_infected_thread(const int32_t *__restrict__ idx,
                                                    const int32_t *__restrict__ sin, int32_t b,
                                                    int32_t e, int32_t ci)
{
    for (int32_t k = b; k < e; ++k)
        if (__ldg(sin + __ldg(idx + k)) == ci) return true;
    return false;
}

__device__ __forceinline__ bool any_infected_warp(const int32_t *__restrict__ idx,
                                                  const int32_t *__restrict__ sin, int32_t b,
                                                  int32_t e, int32_t ci, int lane)
{
    for (int32_t k0 = b; k0 < e; k0 += 32) {
        const int32_t k = k0 + lane;
        const bool hit = (k < e) && (__ldg(sin + __ldg(idx + k)) == ci);
        if (__any_sync(FULL_MASK, hit)) return true;
    }
    return false;
}

// SIR-B: the j-th infected neighbour found draws philox(salt 2 + j); any draw
// below beta infects. Only the number of infected neighbours matters, so the
// warp version counts 32 at a time and tests the next c draws in parallel.
__device__ __forceinline__ bool trials_thread(const int32_t *__restrict__ idx,
                                              const int32_t *__restrict__ sin, int32_t b,
                                              int32_t e, int32_t ci, uint32_t c0b, uint32_t lid,
                                              uint32_t key, uint32_t kinf)
{
    uint32_t j = 0;
    for (int32_t k = b; k < e; ++k) {
        if (__ldg(sin + __ldg(idx + k)) == ci) {
            if (sg_philox_k23(c0b + 2u + j, lid, key) < kinf) return true;
            ++j;
        }
    }
    return false;
}

__device__ __forceinline__ bool trials_warp(const int32_t *__restrict__ idx,
                                            const int32_t *__restrict__ sin, int32_t b, int32_t e,
                                            int32_t ci, uint32_t c0b, uint32_t lid, uint32_t key,
                                            uint32_t kinf, int lane)
{
    uint32_t j = 0;
    for (int32_t k0 = b; k0 < e; k0 += 32) {
        const int32_t k = k0 + lane;
        const bool hit = (k < e) && (__ldg(sin + __ldg(idx + k)) == ci);
        const unsigned m = __ballot_sync(FULL_MASK, hit);
        if (m) {
            const uint32_t c = (uint32_t)__popc(m);
            const bool ok = ((uint32_t)lane < c) &&
                            (sg_philox_k23(c0b + 2u + j + (uint32_t)lane, lid, key) < kinf);
            if (__any_sync(FULL_MASK, ok)) return true;
            j += c;
        }
    }
    return false;
}

template <int VARIANT, bool STATS>
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_pull_kernel(SgTickArgs a)
{
    __shared__ int32_t hubq[SG_SIR_THREADS];
    __shared__ int32_t hubn;
    __shared__ unsigned long long red[4][kWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int32_t *__restrict__ off = a.off;
    const int32_t *__restrict__ idx = a.idx;

    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
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
        unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;

        for (int32_t base = tile.begin; base < tile.end; base += SG_SIR_THREADS) {
            if (tid == 0) hubn = 0;
            __syncthreads();
            const int32_t i = base + tid;
            if (i < tile.end) {
                const int32_t s = sin[i];
                int32_t out = s;
                bool deferred = false;
                if (s == ci) {
                    if (sg_philox_k23(c0b + 1u, seg_lid(sg, i), key) < krec) out = cr;
                } else if (s == cs) {
                    const uint32_t lid = seg_lid(sg, i);
                    if (VARIANT == 1) {
                        const bool lucky = sg_philox_k23(c0b + 1u, lid, key) < kinf;
                        if (lucky || STATS) {
                            const int32_t b = __ldg(off + i), e = __ldg(off + i + 1);
                            if (STATS) eS += (unsigned long long)(e - b);
                            if (lucky) {
                                if (e - b > a.hub_deg) {
                                    deferred = true;
                                    hubq[atomicAdd(&hubn, 1)] = i;
                                } else if (any_infected_thread(idx, sin, b, e, ci)) {
                                    out = ci;
                                }
                            }
                        }
                    } else {
                        const int32_t b = __ldg(off + i), e = __ldg(off + i + 1);
                        if (STATS) eS += (unsigned long long)(e - b);
                        if (e - b > a.hub_deg) {
                            deferred = true;
                            hubq[atomicAdd(&hubn, 1)] = i;
                        } else if (trials_thread(idx, sin, b, e, ci, c0b, lid, key, kinf)) {
                            out = ci;
                        }
                    }
                }
                if (!deferred) {
                    sout[i] = out;
                    if (STATS) {
                        nS += (out == cs);
                        nI += (out == ci);
                        nR += (out == cr);
                    }
                }
            }
            __syncthreads();
            const int nh = hubn;
            for (int q = warp; q < nh; q += kWarps) {
                const int32_t h = hubq[q];
                const int32_t b = __ldg(off + h), e = __ldg(off + h + 1);
                bool inf;
                if (VARIANT == 1)
                    inf = any_infected_warp(idx, sin, b, e, ci, lane);
                else
                    inf = trials_warp(idx, sin, b, e, ci, c0b, seg_lid(sg, h), key, kinf, lane);
                const int32_t out = inf ? ci : cs;
                if (lane == 0) {
                    sout[h] = out;
                    if (STATS) {
                        nS += (out == cs);
                        nI += (out == ci);
                    }
                }
            }
            // the next iteration's hubn reset is ordered after this read by its
            // __syncthreads only if every thread has read hubn: sync here.
            __syncthreads();
        }
        if (STATS && sg.stats) block_flush4(nS, nI, nR, eS, sg.stats + 4 * (int64_t)a.r, red);
    }
}

// ---- count strategy -------------------------------------------------------------
// cnt[i] = number of infected agents in row i. A susceptible agent then needs
// only cnt[i]: SIR-A infects iff cnt > 0 and u < beta, SIR-B iff one of the
// draws salt 2 .. 2+cnt-1 is below beta. Agents whose infected status changed
// this tick are appended to a change list; the scatter kernel then adds +-1 to
// cnt over their transpose rows (the agents that list them as neighbours).

__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_init_kernel(SgTickArgs a)
{
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int par = sg.par0 & 1;
        const int32_t *__restrict__ sin = (const int32_t *)(par ? a.buf1 : a.buf0);
        const int32_t ci = sg.ci;
        // one warp per agent: rows of any length, coalesced
        for (int32_t i = tile.begin + (int32_t)(threadIdx.x >> 5); i < tile.end; i += kWarps) {
            const int32_t b = a.off[i], e = a.off[i + 1];
            int32_t c = 0;
            for (int32_t k = b + lane; k < e; k += 32) c += (sin[a.idx[k]] == ci);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(FULL_MASK, c, o);
            if (lane == 0) a.cnt[i] = c;
        }
    }
}

__device__ __forceinline__ void push_change(int32_t *changes, int32_t *counter, bool has,
                                            int32_t code)
{
    const unsigned m = __ballot_sync(FULL_MASK, has);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(FULL_MASK, base, leader);
    if (has) changes[base + __popc(m & ((1u << lane) - 1u))] = code;
}

template <int VARIANT, bool STATS>
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_step_kernel(SgTickArgs a)
{
    __shared__ unsigned long long red[4][kWarps];
    const int tid = threadIdx.x;
    int32_t *counter = a.nchanges + a.r;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int64_t tick = sg.tick0 + a.r;
        if (tick >= sg.end_tick) continue;
        const int par = (sg.par0 + a.r) & 1;
        const int32_t *__restrict__ sin = (const int32_t *)(par ? a.buf1 : a.buf0);
        int32_t *__restrict__ sout = (int32_t *)(par ? a.buf0 : a.buf1);
        const uint32_t c0b = sg_c0base(tick);
        const uint32_t key = sg.key, kinf = sg.kinf, krec = sg.krec;
        const int32_t cs = sg.cs, ci = sg.ci, cr = sg.cr;
        unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;
        // tile.end - tile.begin is a multiple of the block size except for the
        // segment's last tile; the loop keeps every lane of a warp alive for
        // the ballot in push_change.
        for (int32_t base = tile.begin; base < tile.end; base += SG_SIR_THREADS) {
            const int32_t i = base + tid;
            bool has = false;
            int32_t code = 0;
            if (i < tile.end) {
                const int32_t s = sin[i];
                int32_t out = s;
                if (s == ci) {
                    if (sg_philox_k23(c0b + 1u, seg_lid(sg, i), key) < krec) {
                        out = cr;
                        has = true;
                        code = ~i;
                    }
                } else if (s == cs) {
                    if (STATS) eS += (unsigned long long)(a.off[i + 1] - a.off[i]);
                    const int32_t k = a.cnt[i];
                    if (k > 0) {
                        const uint32_t lid = seg_lid(sg, i);
                        bool inf = false;
                        if (VARIANT == 1) {
                            inf = sg_philox_k23(c0b + 1u, lid, key) < kinf;
                        } else {
                            for (int32_t j = 0; j < k; ++j) {
                                if (sg_philox_k23(c0b + 2u + (uint32_t)j, lid, key) < kinf) {
                                    inf = true;
                                    break;
                                }
                            }
                        }
                        if (inf) {
                            out = ci;
                            has = true;
                            code = i;
                        }
                    }
                }
                sout[i] = out;
                if (STATS) {
                    nS += (out == cs);
                    nI += (out == ci);
                    nR += (out == cr);
                }
            }
            push_change(a.changes, counter, has, code);
        }
        if (STATS && sg.stats) block_flush4(nS, nI, nR, eS, sg.stats + 4 * (int64_t)a.r, red);
    }
}

__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_scatter_kernel(SgTickArgs a)
{
    __shared__ int32_t hubq[SG_SIR_THREADS];
    __shared__ int32_t hubn;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int32_t n = a.nchanges[a.r];
    for (int32_t base = blockIdx.x * SG_SIR_THREADS; base < n; base += gridDim.x * SG_SIR_THREADS) {
        if (tid == 0) hubn = 0;
        __syncthreads();
        const int32_t q = base + tid;
        if (q < n) {
            const int32_t c = a.changes[q];
            const int32_t g = c >= 0 ? c : ~c;
            const int32_t delta = c >= 0 ? 1 : -1;
            const int32_t b = a.toff[g], e = a.toff[g + 1];
            if (e - b > 32) {
                hubq[atomicAdd(&hubn, 1)] = c;
            } else {
                for (int32_t k = b; k < e; ++k) atomicAdd(a.cnt + a.tidx[k], delta);
            }
        }
        __syncthreads();
        const int nh = hubn;
        for (int h = warp; h < nh; h += kWarps) {
            const int32_t c = hubq[h];
            const int32_t g = c >= 0 ? c : ~c;
            const int32_t delta = c >= 0 ? 1 : -1;
            const int32_t b = a.toff[g], e = a.toff[g + 1];
            for (int32_t k = b + lane; k < e; k += 32) atomicAdd(a.cnt + a.tidx[k], delta);
        }
        __syncthreads();
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

cudaError_t sg_launch_sir_count_step(const SgTickArgs &a, int variant, bool stats, int grid,
                                     cudaStream_t st)
{
    if (variant == 1) {
        if (stats)
            sir_count_step_kernel<1, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        else
            sir_count_step_kernel<1, false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    } else {
        if (stats)
            sir_count_step_kernel<2, true><<<grid, SG_SIR_THREADS, 0, st>>>(a);
        else
            sir_count_step_kernel<2, false><<<grid, SG_SIR_THREADS, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t sg_launch_sir_count_scatter(const SgTickArgs &a, int grid, cudaStream_t st)
{
    sir_count_scatter_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t sg_launch_opinion(const SgTickArgs &a, int grid, cudaStream_t st)
{
    opinion_kernel<<<grid, SG_SIR_THREADS, 0, st>>>(a);
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
