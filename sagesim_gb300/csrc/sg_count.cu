// sg_count.cu -- kernels of the count strategy for sm_103a.
//
// The count strategy keeps, for every susceptible agent, the number of its
// infected neighbours (cnt), so a tick reads one agent's own state and count
// instead of its whole CSR row: a step kernel draws and records the agents
// whose infected status changed, and a scatter kernel adds +-1 along their
// transpose rows. Tick semantics are SAGESim's (sagesim/model.py:2306-2408):
// the step reads tick-start values, and the scatter that makes this tick's
// changes visible runs after the step, before the next tick.
#include <algorithm>

#include "sg_device.cuh"

namespace {

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
            const int32_t s = i < tile.end ? sin[i] : INT32_MIN;
            bool medium = false;
            int32_t b = 0, e = 0, c = 0;
            if (s == cs) {
                b = a.off[i];
                e = a.off[i + 1];
                if (e - b > a.mega_row) {
                    c = 1; // counted by a mega block; its activity bit is set conservatively
                } else if (e - b > thread_row_of(a)) {
                    medium = true;
                } else {
                    c = count_thread(a.idx, sin, b, e, ci);
                    a.cnt[i] = c;
                }
            }
            unsigned m = __ballot_sync(FULL_MASK, medium);
            while (m) {
                const int l = __ffs(m) - 1;
                m &= m - 1;
                const int32_t hb = __shfl_sync(FULL_MASK, b, l);
                const int32_t he = __shfl_sync(FULL_MASK, e, l);
                int32_t wc = 0;
                warp_row<0>(a.idx, sin, hb, he, ci, 0, 0, 0, 0, lane, &wc);
                if (lane == l) {
                    a.cnt[i] = wc;
                    c = wc;
                }
            }
            if (a.cls) {
                // class byte of every agent and the activity word of these 32
                // agents (wbase is a multiple of 32 whenever a.cls is set)
                if (i < tile.end) a.cls[i] = (uint8_t)(s == ci ? 1 : s == cs ? 0 : s == sg.cr ? 2 : 3);
                const unsigned word = __ballot_sync(FULL_MASK, s == cs && s != ci && c != 0);
                if (lane == 0) a.amask[wbase >> 5] = word;
            }
        }
    }
}

// Count init by scattering from the infected agents, for a step over every
// agent of a graph with one segment (the usual single-model case). The clear
// pass zeroes the counts and the activity words and writes the class bytes; the
// scatter pass walks the transpose row of each infected agent (one warp per
// infected agent, coalesced) adding 1 to every neighbour's count and setting
// the activity bit of susceptible neighbours. The counts equal the per-row
// scan of sir_count_init_kernel; the work is the infected agents' degree sum
// instead of every row, which at the start of an outbreak is a small fraction.
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_init_clear_kernel(SgTickArgs a)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int32_t *__restrict__ sin = (const int32_t *)((sg.par0 & 1) ? a.buf1 : a.buf0);
        for (int32_t wbase = tile.begin + warp * 32; wbase < tile.end; wbase += SG_SIR_THREADS) {
            const int32_t i = wbase + lane;
            if (i < tile.end) {
                a.cnt[i] = 0;
                if (a.cls) {
                    const int32_t st = sin[i];
                    a.cls[i] = (uint8_t)(st == sg.ci ? 1 : st == sg.cs ? 0 : st == sg.cr ? 2 : 3);
                }
            }
            if (a.cls && lane == 0) a.amask[wbase >> 5] = 0u;
        }
    }
}

__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_init_scatter_kernel(SgTickArgs a)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const SgTile tile = a.tiles[t];
        const SgSeg &sg = a.segs[tile.seg];
        const int32_t *__restrict__ sin = (const int32_t *)((sg.par0 & 1) ? a.buf1 : a.buf0);
        for (int32_t wbase = tile.begin + warp * 32; wbase < tile.end; wbase += SG_SIR_THREADS) {
            const int32_t i = wbase + lane;
            unsigned m = __ballot_sync(FULL_MASK, i < tile.end && sin[i] == sg.ci);
            while (m) {
                const int l = __ffs(m) - 1;
                m &= m - 1;
                const int32_t j = wbase + l;
                const int32_t b = __ldg(a.toff + j), e = __ldg(a.toff + j + 1);
                for (int32_t p = b + lane; p < e; p += 32) {
                    const int32_t k = __ldg(a.tidx + p);
                    atomicAdd(a.cnt + k, 1);
                    if (a.cls && a.cls[k] == 0) atomicOr(a.amask + (k >> 5), 1u << (k & 31));
                }
            }
        }
    }
}

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

// Hybrid count step: whether tick r runs the busy-tick form (flat draws or the
// loop form) instead of the class sweep. The choice reads the change totals of
// the two previous ticks, which every block sees alike. The busy-tick form
// pays a fixed cost per agent, the class sweep one per candidate; while an
// epidemic grows, candidates (susceptible agents next to new infections, often
// clustered around hubs) outnumber changes by far, so the loop form is chosen
// from a lower change count on the way up than on the way down.
__device__ __forceinline__ bool hybrid_loop_tick(const SgTickArgs &a)
{
    if (a.hybrid_rise <= 0 || a.r < 2 || !a.tick_changes) return false;
    const int32_t c1 = a.tick_changes[a.r - 1], c2 = a.tick_changes[a.r - 2];
    return (c1 > a.hybrid_rise && c1 >= c2) || c1 > a.hybrid_fall;
}

// A changed agent whose transpose row is longer than kSegRow is handed to the
// scatter as row segments of kSegRow entries on their own work list, so no
// single warp walks a hub's whole row; the chunk pass skips such rows.
constexpr int32_t kSegRow = SG_SEG_ROW;

// What the scatter needs of changed agent g, whose change-list entry is
// `slot`: a long transpose row goes to the segment list (its recorded row is
// then empty); the row [begin, end) is recorded beside the entry when the
// change-row array is kept, so the scatter does not load the offsets again.
__device__ __forceinline__ void record_changed_row(const SgTickArgs &a, int32_t slot, int32_t g, int32_t delta)
{
    if (!a.change_rows && !a.rowsegs) return;
    const int32_t b = __ldg(a.toff + g), e = __ldg(a.toff + g + 1);
    int32_t re = e;
    if (a.rowsegs && e - b > kSegRow) {
        const int32_t nseg = (e - b + kSegRow - 1) / kSegRow;
        const int32_t base = atomicAdd(a.nrowsegs + a.r, nseg);
        for (int32_t j = 0; j < nseg; ++j) {
            const int32_t sb = b + j * kSegRow;
            a.rowsegs[base + j] = SgRowSeg{sb, min(sb + kSegRow, e), delta, 0};
        }
        re = b;
    }
    if (a.change_rows) a.change_rows[slot] = make_int2(b, re);
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
    if (a.hybrid_rise > 0) {
        if (!hybrid_loop_tick(a)) return; // the class sweep takes this tick
        // activity bits owed a rebuild stay owed until a sweep tick rebuilds them
        if (blockIdx.x == 0 && threadIdx.x == 0 && a.mrebuild && a.mrebuild[a.r]) a.mrebuild[a.r + 1] = 1;
    }
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
                    if (has && a.cls) a.cls[i] = (uint8_t)(code >= 0 ? 1 : 2);
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
                    if (has) {
                        const int32_t slot = pos + __popc(m & ((1u << lane) - 1u));
                        tchanges[slot] = code;
                        record_changed_row(a, tile.begin + slot, i, code >= 0 ? 1 : -1);
                    }
                }
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
                if (a.tick_changes && n > 0) atomicAdd(a.tick_changes + a.r, n);
                if (a.tick_cand) atomicAdd(a.tick_cand + a.r, tile.end - tile.begin);
                if (a.chunks && n > 0) chunk_base = atomicAdd(a.nchunks + a.r, c);
            }
            __syncthreads();
            if (a.chunks && n > 0) {
                const int32_t base = chunk_base;
                for (int32_t j = tid; j < c; j += SG_SIR_THREADS)
                    a.chunks[base + j] = SgChunk{tile.begin + 32 * j, min(32, n - 32 * j)};
            }
        }
        if (STATS && a.segs[tile.seg].stats)
            block_flush4(nS, nI, nR, eS, a.segs[tile.seg].stats + 4 * (int64_t)a.r, red);
        __syncthreads(); // nch is reset by the next tile
    }
}

// Bits 0-3: which of the four class bytes of w equal c (a byte equal to c
// becomes 0xFF under the SIMD compare; the bytes' low bits are gathered by one
// multiply).
__device__ __forceinline__ uint32_t class_mask4(uint32_t w, uint32_t c)
{
    return ((__vcmpeq4(w, c * 0x01010101u) & 0x01010101u) * 0x01020408u) >> 24;
}

// ---- count step, flat draws (busy ticks) -----------------------------------------------
#include "sg_count_flat.cuh"

// ---- count step, class sweep ---------------------------------------------------------
// In-place count step over one-byte agent classes (a.cls: 0 S, 1 I, 2 R,
// 3 other) and activity bits (a.amask: bit i is set whenever cnt[i] may be
// above 0). Only an infected agent (recovery draw) or a susceptible agent whose
// bit is set (count read; infection draws when it is above 0) is a candidate;
// every other agent costs a byte read and a few bit operations, so late in an
// epidemic a tick reads about one byte per agent instead of its state, count
// and RNG key.
//
// A block takes a group of 8 tiles, one warp per tile (group g: tiles g,
// g + G, g + 2G, ... with G groups):
//   1. each warp reads its tile's classes and bits (four 16-byte class loads
//      and four mask half-words per lane) and writes its candidates' slots to
//      its part of shared memory;                                   -- barrier
//   2. the block's threads share the concatenated candidate lists (U = 4 per
//      thread in flight): count and RNG key, the draws (recovery: salt 1;
//      SIR-B infection: salt 2 .. 2+k-1 with early exit; one flattened loop
//      over the thread's candidates), state, class and change-list writes
//      (per-tile shared counters);                                   -- barrier
//   3. each warp publishes its tile's change count and chunks.
// Candidates cluster (an infected hub makes its whole neighbourhood, often a
// few consecutive tiles, candidates at once); spreading consecutive tiles over
// blocks and sharing a group's candidates among its 8 warps keeps such tiles
// from serialising on one warp or block, and a group costs three dependent
// memory round trips and two barriers. A count read as 0 clears its
// bit. In a rebuild tick (the previous scatter did not keep the bits) every
// susceptible agent is a candidate: phase 1 sets the bits of all of them and
// phase 2 clears those whose count is 0.
struct SgSweepTile {
    uint32_t c0b, key, kinf, krec;
    int32_t ci, cr, lid_base, live; // live: the tile's segment ticks this launch
    int32_t begin, pad;
    const uint32_t *lids;
    unsigned long long *stats;
};

// Shared memory of the class sweep with WPT warps per tile.
template <int WPT>
struct SgSweepSmem {
    uint16_t cand[kWarps][SG_TILE]; // slot | infected << 11
    SgSweepTile tp[kWarps];
    int32_t ccount[kWarps], nch[kWarps / WPT];
    unsigned long long dstat[kWarps][3]; // per warp region: S, I, R changes (mod 2^64)
};

// One tick of the class sweep over the launch's tiles (the caller has decided
// that this form takes the tick).
template <int VARIANT, bool STATS, int WPT>
__device__ __forceinline__ void sweep_tick(const SgTickArgs &a, SgSweepSmem<WPT> &sm)
{
    constexpr int kRun = 16;                     // agents per lane and class load
    constexpr int kRuns = SG_TILE / (32 * kRun); // runs of a whole tile per lane
    constexpr int kMyRuns = kRuns / WPT;         // runs of this warp's part of a tile
    constexpr int TPB = kWarps / WPT;            // tiles per block (group)
    constexpr int U = 2;                         // candidates per thread in flight (2: less divergence than 4)
    static_assert(kRuns * 32 * kRun == SG_TILE, "runs must cover the tile");
    static_assert(kMyRuns * WPT == kRuns && TPB * WPT == kWarps, "warps must split tiles evenly");
    static_assert(SG_TILE <= 0x800, "slot must fit in 11 bits");
    auto &sh_cand = sm.cand;
    auto &sh_tp = sm.tp;
    auto &sh_ccount = sm.ccount;
    auto &sh_nch = sm.nch;
    auto &sh_dstat = sm.dstat;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ti = warp / WPT, part = warp % WPT; // this warp's tile in the group and part of it
    int32_t *const state = (int32_t *)a.buf0;
    const bool rebuild = a.mrebuild && a.mrebuild[a.r];
    const int32_t ngroups = (a.ntiles + TPB - 1) / TPB;
    int32_t cur_seg = -1; // this warp's cached segment
    SgSweepTile my{};
    if (tid < TPB) sh_nch[tid] = 0;
    for (int32_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
        // 1. this warp's part of its tile: classes and bits -> candidate list
        // tiles of a group are ngroups apart, so a cluster of candidate-dense
        // consecutive tiles (a hub's neighbourhood) is spread over TPB blocks
        const int32_t t = ti * ngroups + g;
        int32_t C = 0;
        unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;
        if (t < a.ntiles) {
            const SgTile tile = a.tiles[t];
            if (tile.seg != cur_seg) {
                const SgSeg &sg = a.segs[tile.seg];
                cur_seg = tile.seg;
                const int64_t tick = sg.tick0 + a.r;
                my.c0b = sg_c0base(tick);
                my.key = sg.key;
                my.kinf = sg.kinf;
                my.krec = sg.krec;
                my.ci = sg.ci;
                my.cr = sg.cr;
                my.lid_base = sg.lid_base;
                my.live = tick < sg.end_tick;
                my.lids = sg.lids;
                my.stats = sg.stats;
            }
            my.begin = tile.begin;
            if (my.live) {
                uint16_t *const wcand = sh_cand[warp];
                uint32_t cm[kMyRuns], im[kMyRuns];
#pragma unroll
                for (int rr = 0; rr < kMyRuns; ++rr) {
                    const int r = part * kMyRuns + rr;
                    const int32_t b = tile.begin + r * (32 * kRun) + lane * kRun;
                    const int32_t nv = min(kRun, tile.end - b);
                    uint32_t w[4] = {0x03030303u, 0x03030303u, 0x03030303u, 0x03030303u};
                    if (nv == kRun) {
                        const uint4 v = *reinterpret_cast<const uint4 *>(a.cls + b);
                        w[0] = v.x;
                        w[1] = v.y;
                        w[2] = v.z;
                        w[3] = v.w;
                    } else if (nv > 0) {
#pragma unroll
                        for (int e = 0; e < kRun; ++e)
                            if (e < nv) {
                                const int sh = 8 * (e & 3);
                                w[e >> 2] = (w[e >> 2] & ~(0xFFu << sh)) | ((uint32_t)a.cls[b + e] << sh);
                            }
                    }
                    const uint32_t bits = nv > 0 ? (a.amask[b >> 5] >> (b & 31)) & 0xFFFFu : 0u;
                    // class bytes compared four at a time: bit e of each mask is agent e
                    uint32_t sm = 0, imr = 0, rm = 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        sm |= class_mask4(w[q], 0u) << (4 * q);
                        imr |= class_mask4(w[q], 1u) << (4 * q);
                        if (STATS) rm |= class_mask4(w[q], 2u) << (4 * q);
                    }
                    if (rebuild) {
                        // lanes 2j and 2j + 1 hold the 32 agents of one mask word
                        uint32_t word = sm << (b & 31);
                        word |= __shfl_xor_sync(FULL_MASK, word, 1);
                        if (!(lane & 1) && nv > 0) a.amask[b >> 5] = word;
                    }
                    cm[rr] = (rebuild ? sm : (sm & bits)) | imr;
                    im[rr] = imr;
                    if (STATS) {
                        nS += __popc(sm);
                        nI += __popc(imr);
                        nR += __popc(rm);
                        for (uint32_t m = sm; m; m &= m - 1) {
                            const int32_t i = b + __ffs(m) - 1;
                            eS += (unsigned long long)(__ldg(a.off + i + 1) - __ldg(a.off + i));
                        }
                    }
                }
                int32_t mine = 0;
#pragma unroll
                for (int rr = 0; rr < kMyRuns; ++rr) mine += __popc(cm[rr]);
                int32_t x = mine;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int32_t y = __shfl_up_sync(FULL_MASK, x, o);
                    if (lane >= o) x += y;
                }
                C = __shfl_sync(FULL_MASK, x, 31);
                int32_t pos = x - mine;
#pragma unroll
                for (int rr = 0; rr < kMyRuns; ++rr)
                    for (uint32_t m = cm[rr]; m; m &= m - 1) {
                        const int e = __ffs(m) - 1;
                        const int r = part * kMyRuns + rr;
                        wcand[pos++] = (uint16_t)((r * (32 * kRun) + lane * kRun + e) | (((im[rr] >> e) & 1u) << 11));
                    }
            }
        }
        if (lane == 0) {
            sh_ccount[warp] = C;
            if (a.tick_cand && C > 0) atomicAdd(a.tick_cand + a.r, C);
            SgSweepTile tp = my;
            tp.live = (t < a.ntiles) && my.live;
            sh_tp[warp] = tp;
            if (STATS) {
                sh_dstat[warp][0] = 0;
                sh_dstat[warp][1] = 0;
                sh_dstat[warp][2] = 0;
            }
        }
        __syncthreads();
        // 2. the group's candidates, shared by all threads
        int32_t pre[kWarps + 1];
        pre[0] = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) pre[w + 1] = pre[w] + sh_ccount[w];
        const int32_t total = pre[kWarps];
        for (int32_t q0 = 0; q0 < total; q0 += SG_SIR_THREADS * U) {
            int32_t gi[U], kk[U], tw[U];
            uint32_t ll[U];
            bool infk[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int32_t q = q0 + u * SG_SIR_THREADS + tid;
                int32_t w = 0; // region of q: the last w with pre[w] <= q
#pragma unroll
                for (int v = 1; v < kWarps; ++v) w += (pre[v] <= q);
                tw[u] = w;
                gi[u] = -1;
                kk[u] = 0;
                ll[u] = 0;
                infk[u] = false;
                if (q < total) {
                    const uint32_t ent = sh_cand[w][q - pre[w]];
                    const int32_t i = sh_tp[w].begin + (int32_t)(ent & 0x7FFu);
                    gi[u] = i;
                    infk[u] = (ent >> 11) != 0;
                    if (!infk[u]) kk[u] = a.cnt[i];
                    const uint32_t *lids = sh_tp[w].lids;
                    ll[u] = lids ? __ldg(lids + i) : (uint32_t)(i - sh_tp[w].lid_base);
                }
            }
            // draws: one flattened loop over this thread's candidates (counter
            // c0[u] + j, j < nd[u], until a hit), so a warp runs as long as its
            // busiest thread's total draws rather than the sum of per-slot maxima
            int32_t nd[U];
            uint32_t c0[U], thr[U], kkey[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                nd[u] = 0;
                c0[u] = thr[u] = kkey[u] = 0;
                const int32_t i = gi[u];
                if (i < 0) continue;
                const SgSweepTile &tp = sh_tp[tw[u]];
                kkey[u] = tp.key;
                if (infk[u]) {
                    nd[u] = 1;
                    c0[u] = tp.c0b + 1u;
                    thr[u] = tp.krec;
                } else if (kk[u] > 0) {
                    nd[u] = VARIANT == 1 ? 1 : kk[u];
                    c0[u] = tp.c0b + (VARIANT == 1 ? 1u : 2u);
                    thr[u] = tp.kinf;
                } else {
                    atomicAnd(a.amask + (i >> 5), ~(1u << (i & 31)));
                }
            }
            uint32_t hitm = 0;
            int cur = -1;
            int32_t left = 0;
            uint32_t cc = 0, cl = 0, ct = 0, ckey = 0;
            auto next = [&](int from) {
                cur = -1;
#pragma unroll
                for (int v = U - 1; v >= 0; --v)
                    if (v >= from && nd[v] > 0) cur = v;
#pragma unroll
                for (int v = 0; v < U; ++v)
                    if (v == cur) {
                        left = nd[v];
                        cc = c0[v];
                        cl = ll[v];
                        ct = thr[v];
                        ckey = kkey[v];
                    }
            };
            next(0);
            while (cur >= 0) {
                const bool h = sg_philox_k23(cc, cl, ckey) < ct;
                ++cc;
                if (h) {
                    hitm |= 1u << cur;
                    next(cur + 1);
                } else if (--left == 0) {
                    next(cur + 1);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (!((hitm >> u) & 1u)) continue;
                const int32_t i = gi[u];
                const SgSweepTile &tp = sh_tp[tw[u]];
                state[i] = infk[u] ? tp.cr : tp.ci;
                a.cls[i] = (uint8_t)(infk[u] ? 2 : 1);
                const int32_t p = atomicAdd(&sh_nch[tw[u] / WPT], 1);
                a.changes[tp.begin + p] = infk[u] ? ~i : i;
                record_changed_row(a, tp.begin + p, i, infk[u] ? -1 : 1);
                if (STATS) {
                    // S -> I: S - 1, I + 1; I -> R: I - 1, R + 1 (sums mod 2^64)
                    atomicAdd(&sh_dstat[tw[u]][infk[u] ? 1 : 0], ~0ull);
                    atomicAdd(&sh_dstat[tw[u]][infk[u] ? 2 : 1], 1ull);
                }
            }
        }
        __syncthreads();
        // 3. the tile's change count and chunks (its first warp), statistics (every warp)
        if (t < a.ntiles && part == 0) {
            const int32_t n = sh_nch[ti];
            if (lane == 0) {
                a.tile_nch[t] = n;
                if (a.tick_changes && n > 0) atomicAdd(a.tick_changes + a.r, n);
            }
            if (a.chunks && n > 0) {
                const int32_t c = (n + 31) >> 5;
                int32_t cb = 0;
                if (lane == 0) cb = atomicAdd(a.nchunks + a.r, c);
                cb = __shfl_sync(FULL_MASK, cb, 0);
                for (int32_t j = lane; j < c; j += 32) a.chunks[cb + j] = SgChunk{my.begin + 32 * j, min(32, n - 32 * j)};
            }
        }
        if (t < a.ntiles) {
            if (STATS && my.live && my.stats) {
                const unsigned long long v0 = warp_sum(nS), v1 = warp_sum(nI), v2 = warp_sum(nR),
                                         v3 = warp_sum(eS);
                if (lane == 0) {
                    unsigned long long *dst = my.stats + 4 * (int64_t)a.r;
                    atomicAdd(dst, v0 + sh_dstat[warp][0]);
                    atomicAdd(dst + 1, v1 + sh_dstat[warp][1]);
                    atomicAdd(dst + 2, v2 + sh_dstat[warp][2]);
                    atomicAdd(dst + 3, v3);
                }
            }
        }
        __syncwarp();
        if (lane == 0 && part == 0) sh_nch[ti] = 0; // read above by this warp only
    }
}

template <int VARIANT, bool STATS, int WPT>
__global__ void __launch_bounds__(SG_SIR_THREADS, 5) sir_count_sweep_kernel(SgTickArgs a)
{
    __shared__ SgSweepSmem<WPT> sm;
    if (hybrid_loop_tick(a)) return; // the loop form takes this tick
    sweep_tick<VARIANT, STATS, WPT>(a, sm);
}

// The hybrid step with flat draws in one launch: the class sweep in quiet
// ticks and flat draws in busy ones (hybrid_loop_tick gives every block the
// same answer), so no idle kernel is launched per tick. Shared memory is the
// larger of the two forms' (they never run in the same launch).
template <int WPT>
union SgHybridSmem {
    SgSweepSmem<WPT> sweep;
    SgFlatSmem flat;
};

template <int VARIANT, bool STATS, int WPT>
__global__ void __launch_bounds__(SG_SIR_THREADS, kFlatBlocksPerSm) sir_count_hybrid_kernel(SgTickArgs a)
{
    __shared__ SgHybridSmem<WPT> sm;
    if (hybrid_loop_tick(a)) flat_tick<VARIANT, STATS>(a, sm.flat);
    else sweep_tick<VARIANT, STATS, WPT>(a, sm.sweep);
}

// ---- scatter -------------------------------------------------------------------------
// +-1 along the transpose rows of up to 32 changes, one per lane (b, e: the
// lane's row; empty for no change).

// cnt[d] += delta; with set_bits a +1 also marks d active for the class sweep.
__device__ __forceinline__ void count_add(const SgTickArgs &a, int32_t d, int32_t delta, bool set_bits)
{
    atomicAdd(a.cnt + d, delta);
    if (set_bits && delta > 0) atomicOr(a.amask + (d >> 5), 1u << (d & 31));
}

// Whether this tick's scatter keeps the activity bits. Setting a bit on every
// +1 costs one more atomic per transpose entry; when more than one agent in 32
// changed this tick (the epidemic's peak, when most susceptible agents have
// infected neighbours anyway), rebuilding the bits in the next sweep (which
// then reads every susceptible agent's count) is cheaper, and the scatter
// flags that instead. Every block reaches the same decision.
__device__ __forceinline__ bool scatter_sets_bits(const SgTickArgs &a)
{
    if (!a.amask) return false;
    if (!a.mrebuild || !a.tick_changes) return true;
    const bool keep = a.tick_changes[a.r] <= a.ntiles * (SG_TILE / 32);
    if (!keep && blockIdx.x == 0 && threadIdx.x == 0) a.mrebuild[a.r + 1] = 1;
    return keep;
}

// Lane-per-row form: a lane walks its own row with 4 independent index loads
// per step; rows longer than thread_row are walked by the whole warp.
__device__ __forceinline__ void scatter_rows_lane(const SgTickArgs &a, int32_t b, int32_t e, int32_t delta,
                                                  int lane, bool sb)
{
    const bool long_row = e - b > thread_row_of(a);
    if (!long_row) {
        for (int32_t k = b; k < e; k += 4) {
            const int32_t last = e - 1;
            const int32_t d0 = __ldg(a.tidx + k);
            const int32_t d1 = __ldg(a.tidx + min(k + 1, last));
            const int32_t d2 = __ldg(a.tidx + min(k + 2, last));
            const int32_t d3 = __ldg(a.tidx + min(k + 3, last));
            count_add(a, d0, delta, sb);
            if (k + 1 < e) count_add(a, d1, delta, sb);
            if (k + 2 < e) count_add(a, d2, delta, sb);
            if (k + 3 < e) count_add(a, d3, delta, sb);
        }
    }
    unsigned m = __ballot_sync(FULL_MASK, long_row);
    while (m) {
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const int32_t hb = __shfl_sync(FULL_MASK, b, l);
        const int32_t he = __shfl_sync(FULL_MASK, e, l);
        const int32_t hd = __shfl_sync(FULL_MASK, delta, l);
        for (int32_t k = hb + lane; k < he; k += 32) count_add(a, __ldg(a.tidx + k), hd, sb);
    }
}

// Load-balanced form: the 32 rows are laid end to end (warp inclusive scan of
// their lengths) and the warp walks the concatenation one entry per lane per
// step, kScatterUnroll steps per round so that each lane has that many
// independent index loads in flight. The row holding entry p is the lane
// whose inclusive sum is the first above p (5-step search over shuffles).
// No lane idles while another finishes a longer row.
constexpr int kScatterUnroll = 4;

__device__ __forceinline__ void scatter_rows_lb(const SgTickArgs &a, int32_t b, int32_t e, int32_t delta, int lane,
                                                bool sb)
{
    const int32_t len = e - b;
    int32_t incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    const int32_t total = __shfl_sync(FULL_MASK, incl, 31);
    const int32_t start = b - (incl - len); // entry p of this lane's row is tidx[start + p]
    for (int32_t p0 = 0; p0 < total; p0 += 32 * kScatterUnroll) {
        int32_t d[kScatterUnroll], dl[kScatterUnroll];
#pragma unroll
        for (int u = 0; u < kScatterUnroll; ++u) {
            const int32_t p = p0 + u * 32 + lane;
            int32_t lo = 0; // lanes whose inclusive sum is <= p (at most 31 while p < total)
#pragma unroll
            for (int w = 16; w >= 1; w >>= 1)
                if (__shfl_sync(FULL_MASK, incl, lo + w - 1) <= p) lo += w;
            const int32_t row0 = __shfl_sync(FULL_MASK, start, lo);
            dl[u] = __shfl_sync(FULL_MASK, delta, lo);
            d[u] = p < total ? __ldg(a.tidx + row0 + p) : -1;
        }
#pragma unroll
        for (int u = 0; u < kScatterUnroll; ++u)
            if (d[u] >= 0) count_add(a, d[u], dl[u], sb);
    }
}

// One warp's 32 changes (entries q0 .. q0 + 31 of the list at `first`, n in
// all). With the change-row array the entry and its row are two independent
// loads; without it the row's offsets are loaded after the entry.
template <bool LB>
__device__ __forceinline__ void scatter_changes(const SgTickArgs &a, int32_t first, int32_t q0, int32_t n, int lane,
                                                bool sb)
{
    const int32_t q = q0 + lane;
    const bool valid = q < n;
    const int32_t c = valid ? a.changes[first + q] : 0;
    const int32_t delta = c >= 0 ? 1 : -1;
    int32_t b = 0, e = 0;
    if (valid) {
        if (a.change_rows) {
            const int2 row = a.change_rows[first + q];
            b = row.x;
            e = row.y;
        } else {
            const int32_t g = c >= 0 ? c : ~c;
            b = __ldg(a.toff + g);
            e = __ldg(a.toff + g + 1);
        }
    }
    if (a.rowsegs && e - b > kSegRow) e = b; // handled through the row-segment list
    if (LB)
        scatter_rows_lb(a, b, e, delta, lane, sb);
    else
        scatter_rows_lane(a, b, e, delta, lane, sb);
}

// One long-row segment (kSegRow entries) by one warp.
__device__ __forceinline__ void scatter_row_segment(const SgTickArgs &a, const SgRowSeg &sgm, int lane, bool sb)
{
    for (int32_t k0 = sgm.begin; k0 < sgm.end; k0 += 32 * kScatterUnroll) {
        int32_t d[kScatterUnroll];
#pragma unroll
        for (int u = 0; u < kScatterUnroll; ++u) {
            const int32_t k = k0 + u * 32 + lane;
            d[u] = k < sgm.end ? __ldg(a.tidx + k) : -1;
        }
#pragma unroll
        for (int u = 0; u < kScatterUnroll; ++u)
            if (d[u] >= 0) count_add(a, d[u], sgm.delta, sb);
    }
}

// The tick's long-row segments, one per warp.
__device__ __forceinline__ void scatter_row_segments(const SgTickArgs &a, int lane, int warp_id, int nwarps, bool sb)
{
    const int32_t nsg = a.nrowsegs[a.r];
    for (int32_t w = warp_id; w < nsg; w += nwarps) scatter_row_segment(a, a.rowsegs[w], lane, sb);
}

// Work-list form: warps take the tick's non-empty 32-change chunks, so a tile
// with thousands of changes is spread over many warps, and then the long-row
// segments, as one list (segments continue where the chunks end, so the warps
// that took chunks are not also the ones that take the segments).
template <bool LB>
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_scatter_chunks_kernel(SgTickArgs a)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int32_t nck = a.nchunks[a.r];
    const int32_t nitems = nck + (a.rowsegs ? a.nrowsegs[a.r] : 0);
    const bool sb = scatter_sets_bits(a);
    for (int32_t w = blockIdx.x * kWarps + warp; w < nitems; w += gridDim.x * kWarps) {
        if (w < nck) {
            const SgChunk ck = a.chunks[w];
            scatter_changes<LB>(a, ck.first, 0, ck.count, lane, sb);
        } else {
            scatter_row_segment(a, a.rowsegs[w - nck], lane, sb);
        }
    }
}

// Per-tile form (no work list): blocks walk the tiles and their warps the
// tile's changes.
template <bool LB>
__global__ void __launch_bounds__(SG_SIR_THREADS) sir_count_scatter_kernel(SgTickArgs a)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool sb = a.amask != nullptr; // no change total here: the bits are always kept
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const int32_t n = a.tile_nch[t];
        if (n == 0) continue;
        const int32_t first = a.tiles[t].begin;
        for (int32_t q0 = warp * 32; q0 < n; q0 += SG_SIR_THREADS) scatter_changes<LB>(a, first, q0, n, lane, sb);
    }
    if (a.rowsegs) scatter_row_segments(a, lane, blockIdx.x * kWarps + warp, gridDim.x * kWarps, sb);
}

} // namespace

// Launches kernel k(a), with an L2 access-policy window over the counts when
// a.cnt_window is set: the scatter's random +-1 updates and the steps' count
// reads then find cnt in L2 instead of competing with the streamed arrays.
// (Programmatic dependent launch between the step and scatter kernels was
// measured on the 10^7-agent run: no gain, and a loss next to the class
// sweep's five blocks per SM, so kernels are serialised in stream order.)
static void launch_count_kernel(void (*k)(SgTickArgs), const SgTickArgs &a, int grid, cudaStream_t st)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(SG_SIR_THREADS);
    cfg.stream = st;
    cudaLaunchAttribute at{};
    if (a.cnt_window) {
        at.id = cudaLaunchAttributeAccessPolicyWindow;
        at.val.accessPolicyWindow.base_ptr = a.cnt;
        at.val.accessPolicyWindow.num_bytes = a.cnt_window;
        at.val.accessPolicyWindow.hitRatio = 1.0f;
        at.val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        at.val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = &at;
        cfg.numAttrs = 1;
    }
    cudaLaunchKernelEx(&cfg, k, a);
}

cudaError_t sg_launch_sir_count_init(const SgTickArgs &a, int grid, cudaStream_t st)
{
    launch_count_kernel(sir_count_init_kernel, a, grid, st);
    return cudaGetLastError();
}

cudaError_t sg_launch_sir_count_init_scatter(const SgTickArgs &a, int grid, cudaStream_t st)
{
    launch_count_kernel(sir_count_init_clear_kernel, a, grid, st);
    launch_count_kernel(sir_count_init_scatter_kernel, a, grid, st);
    return cudaGetLastError();
}

template <int V, bool P>
static void count_step_flavour(const SgTickArgs &a, int flavour, int grid, cudaStream_t st)
{
    const bool per8 = flavour & SG_FLAVOUR_PER8, lazy = flavour & SG_FLAVOUR_LAZY;
    const bool dense = V == 2 && (flavour & SG_FLAVOUR_DENSE);
#define SG_CF(N, D, L) launch_count_kernel(sir_count_step_kernel<V, false, P, N, D, L>, a, grid, st)
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

// Grid of the flat-draw (and merged hybrid) launches: three blocks per resident
// slot of the current device, at most `grid`; 0 when the device is unknown.
static int flat_grid(int grid)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return 0;
    return std::max(1, std::min(grid, 3 * kFlatBlocksPerSm * sms));
}

cudaError_t sg_launch_sir_count_step(const SgTickArgs &args, int variant, bool stats, bool inplace,
                                     int grid, cudaStream_t st, int *nlaunched)
{
    SgTickArgs a = args;
    if (nlaunched) *nlaunched = 1;
    const bool sweep = (a.flavour & SG_FLAVOUR_SWEEP) && inplace && a.cls && a.chunks;
    if (!sweep) a.hybrid_rise = 0; // the loop form takes every tick
    if (sweep && a.hybrid_rise > 0 && (a.flavour & SG_FLAVOUR_FLAT)) {
        // sweep and flat draws in one launch; the grid is the flat form's (three
        // blocks per resident slot), the sweep's groups are spread over it
        const int wpt = a.sweep_wpt == 2 || a.sweep_wpt == 4 ? a.sweep_wpt : 1;
        const int hgrid = flat_grid(grid);
        if (hgrid <= 0) return cudaErrorInvalidDevice;
#define SG_HY(V, S, W) launch_count_kernel(sir_count_hybrid_kernel<V, S, W>, a, hgrid, st)
#define SG_HYW(V, S) (wpt == 1 ? SG_HY(V, S, 1) : wpt == 2 ? SG_HY(V, S, 2) : SG_HY(V, S, 4))
        if (variant == 1) {
            if (stats) SG_HYW(1, true); else SG_HYW(1, false);
        } else {
            if (stats) SG_HYW(2, true); else SG_HYW(2, false);
        }
#undef SG_HYW
#undef SG_HY
        return cudaGetLastError();
    }
    if (sweep) {
        const int wpt = a.sweep_wpt == 2 || a.sweep_wpt == 4 ? a.sweep_wpt : 1;
        const int tpb = kWarps / wpt;
        const int sgrid = std::max(1, std::min(grid, (a.ntiles + tpb - 1) / tpb)); // one group of tpb tiles per block
#define SG_SW(V, S, W) launch_count_kernel(sir_count_sweep_kernel<V, S, W>, a, sgrid, st)
#define SG_SWW(V, S) (wpt == 1 ? SG_SW(V, S, 1) : wpt == 2 ? SG_SW(V, S, 2) : SG_SW(V, S, 4))
        if (variant == 1) {
            if (stats) SG_SWW(1, true); else SG_SWW(1, false);
        } else {
            if (stats) SG_SWW(2, true); else SG_SWW(2, false);
        }
#undef SG_SWW
#undef SG_SW
        const cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess || a.hybrid_rise <= 0) return err;
        if (nlaunched) *nlaunched = 2;
        // hybrid: the busy-tick form too (it returns at once in sweep ticks)
    }
    if ((a.flavour & SG_FLAVOUR_FLAT) && inplace && a.chunks) {
        // flat draws take the busy ticks (or every tick without the hybrid); a
        // few blocks per resident slot balance tiles of unequal cost better than
        // one wave of many-tile blocks or a block per tile
        grid = flat_grid(grid);
        if (grid <= 0) return cudaErrorInvalidDevice;
        if (variant == 1) {
            if (stats) launch_count_kernel(sir_count_flat_kernel<1, true>, a, grid, st);
            else launch_count_kernel(sir_count_flat_kernel<1, false>, a, grid, st);
        } else {
            if (stats) launch_count_kernel(sir_count_flat_kernel<2, true>, a, grid, st);
            else launch_count_kernel(sir_count_flat_kernel<2, false>, a, grid, st);
        }
        return cudaGetLastError();
    }
    if (stats) { // statistics runs of the loop form use one flavour
        if (variant == 1) {
            if (inplace) launch_count_kernel(sir_count_step_kernel<1, true, true, 4, false, true>, a, grid, st);
            else launch_count_kernel(sir_count_step_kernel<1, true, false, 4, false, true>, a, grid, st);
        } else {
            if (inplace) launch_count_kernel(sir_count_step_kernel<2, true, true, 4, true, true>, a, grid, st);
            else launch_count_kernel(sir_count_step_kernel<2, true, false, 4, true, true>, a, grid, st);
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

cudaError_t sg_launch_sir_count_scatter(const SgTickArgs &args, int grid, cudaStream_t st)
{
    SgTickArgs a = args;
    if (!(a.flavour & SG_FLAVOUR_SWEEP)) a.amask = nullptr; // only the class sweep reads the bits
    const bool lb = !(a.flavour & SG_FLAVOUR_ROWSCATTER);
    if (a.chunks) {
        if (lb) launch_count_kernel(sir_count_scatter_chunks_kernel<true>, a, grid, st);
        else launch_count_kernel(sir_count_scatter_chunks_kernel<false>, a, grid, st);
    } else {
        if (lb) launch_count_kernel(sir_count_scatter_kernel<true>, a, grid, st);
        else launch_count_kernel(sir_count_scatter_kernel<false>, a, grid, st);
    }
    return cudaGetLastError();
}
