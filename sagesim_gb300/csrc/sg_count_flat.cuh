// sg_count_flat.cuh -- the count strategy's flat-draw step for busy ticks.
// Included by sg_count.cu inside its anonymous namespace, after the helpers it
// uses (hybrid_loop_tick, record_changed_row, warp_draws).
//
// Near an epidemic's peak most agents draw: an infected agent one recovery draw
// (salt 1), a susceptible agent with k infected neighbours k infection draws
// (SIR-B: salt 2 .. 2+k-1; SIR-A: one, salt 1). Giving each thread a fixed set
// of agents makes a warp run as long as its busiest lane. Here each warp lays
// the draws of its 256 agents' candidates end to end (a warp scan of the
// per-lane draw counts) and every lane evaluates an equal, contiguous share of
// that sequence: it finds the owner of its first draw by a binary search over
// the candidates' draw ends in the warp's part of shared memory and walks forward,
// four Philox chains in flight. The draws of one candidate may be split
// between lanes; all are evaluated (the outcome depends only on whether some
// draw j < k is below beta, so no order or early exit is needed). Hits are
// bits in shared memory. Draws beyond kFlatCap of one candidate (hubs
// surrounded by infected agents) are done afterwards, warp-wide, only for
// those candidates still without a hit. The warp then lists its changed
// agents in shared memory and each lane applies every 32nd transition exactly
// as the loop form does: state in place, class byte, change-list entry and
// row. Warps balance their own draws and need no
// block barrier until the tile's change count is published; each warp's
// changes go to its own 256-entry part of the tile's change list, announced to
// the scatter as chunks of at most 32 (so this form needs the chunk list).
//
// Lane l of warp w owns the 8 consecutive agents tile.begin + 256 w + 8 l ..
// + 7, read as one 8-byte class load (or two 16-byte state loads without class
// bytes), two 16-byte count loads and two 16-byte key loads issued together.
constexpr int32_t kFlatCap = 32;
constexpr int kFlatBlocksPerSm = 5;            // resident blocks: 48 registers, 33 KB shared memory each
constexpr int kFlatPer = SG_TILE / SG_SIR_THREADS;
constexpr int kFlatIlp = 4;                    // draws a lane evaluates side by side
constexpr int kFlatWarpAgents = 32 * kFlatPer; // agents (and at most candidates) per warp
static_assert(kFlatPer == 8, "the flat step gives each lane 8 agents of a tile");

// U independent Philox streams at once (the same rounds as sg_philox_k23_keys):
// the round chains of one draw are strictly sequential, so a lane keeps U of
// them in flight to hide the multiply and xor latencies.
template <int U>
__device__ __forceinline__ void philox_k23_ilp(uint32_t (&c0)[U], uint32_t (&c1)[U], const SgPhiloxKeys &ks)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t p = (uint64_t)c0[u] * SG_PHILOX_M;
            c0[u] = (uint32_t)(p >> 32) ^ ks.k[r] ^ c1[u];
            c1[u] = (uint32_t)p;
        }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) c0[u] &= 0x7FFFFFu;
}

// Shared memory of the flat step, per warp: one 16-byte record per candidate
// (Philox counter base: the counter of draw d is base + d; RNG key; threshold;
// end of its draws in the warp's sequence | agent 0..255 << 16, so advancing to
// the next candidate is one load) and a hit bit per agent.
struct SgFlatSmem {
    uint4 rec[kWarps][kFlatWarpAgents];
    uint32_t hit[kWarps][kFlatWarpAgents / 32];
    int32_t nw[kWarps], coff[kWarps], cbase;
    unsigned long long red[4][kWarps];
};

// One tick of flat draws over the launch's tiles (the caller has decided that
// this form takes the tick).
template <int VARIANT, bool STATS>
__device__ __forceinline__ void flat_tick(const SgTickArgs &a, SgFlatSmem &sm)
{
    // activity bits owed a rebuild stay owed until a sweep tick rebuilds them
    if (a.hybrid_rise > 0 && blockIdx.x == 0 && threadIdx.x == 0 && a.mrebuild && a.mrebuild[a.r])
        a.mrebuild[a.r + 1] = 1;
    auto &sh_rec = sm.rec;
    auto &sh_hit = sm.hit;
    auto &sh_nw = sm.nw;
    auto &sh_coff = sm.coff;
    auto &sh_cbase = sm.cbase;
    auto &red = sm.red;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int32_t cur_seg = -1;
    int64_t tick = 0, end_tick = 0;
    uint32_t c0b = 0, key = 0, kinf = 0, krec = 0;
    int32_t cs = 0, ci = 0, cr = 0, lid_base = 0;
    const uint32_t *lids = nullptr;
    SgPhiloxKeys ks = sg_philox_keys(0);
    int32_t *const state = (int32_t *)a.buf0; // updated in place
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
            lids = sg.lids;
            lid_base = sg.lid_base;
        }
        if (tick >= end_tick) { // the same for the whole block
            if (tid == 0) a.tile_nch[t] = 0;
            continue;
        }
        const int32_t wfirst = tile.begin + warp * kFlatWarpAgents; // this warp's first agent and list entry
        const int32_t b0 = tile.begin + tid * kFlatPer;
        const bool fast = b0 + kFlatPer <= tile.end && (b0 & 7) == 0; // whole, 32-byte aligned run
        // 1. classes (byte e of cw: 0 S, 1 I, 2 R, 3 other or outside the tile),
        //    counts and RNG keys of this lane's agents. In the aligned case the
        //    three are independent loads issued together (one memory round trip);
        //    counts and keys are needed by most agents of a busy tick anyway.
        unsigned long long cw = 0x0303030303030303ull;
        int32_t k[kFlatPer];
        uint32_t l[kFlatPer];
        if (fast) {
            int4 c0, c1;
            uint4 l0 = make_uint4(0, 0, 0, 0), l1 = l0;
            if (a.cls) cw = *reinterpret_cast<const unsigned long long *>(a.cls + b0);
            c0 = *reinterpret_cast<const int4 *>(a.cnt + b0);
            c1 = *reinterpret_cast<const int4 *>(a.cnt + b0 + 4);
            if (lids) {
                l0 = __ldg(reinterpret_cast<const uint4 *>(lids + b0));
                l1 = __ldg(reinterpret_cast<const uint4 *>(lids + b0 + 4));
            }
            if (!a.cls) {
                const int4 v0 = *reinterpret_cast<const int4 *>(state + b0);
                const int4 v1 = *reinterpret_cast<const int4 *>(state + b0 + 4);
                const int32_t sv[kFlatPer] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
                cw = 0;
#pragma unroll
                for (int e = 0; e < kFlatPer; ++e) {
                    const unsigned long long c = sv[e] == ci ? 1u : sv[e] == cs ? 0u : sv[e] == cr ? 2u : 3u;
                    cw |= c << (8 * e);
                }
            }
            k[0] = c0.x, k[1] = c0.y, k[2] = c0.z, k[3] = c0.w, k[4] = c1.x, k[5] = c1.y, k[6] = c1.z, k[7] = c1.w;
            if (lids) {
                l[0] = l0.x, l[1] = l0.y, l[2] = l0.z, l[3] = l0.w, l[4] = l1.x, l[5] = l1.y, l[6] = l1.z, l[7] = l1.w;
            } else {
#pragma unroll
                for (int e = 0; e < kFlatPer; ++e) l[e] = (uint32_t)(b0 + e - lid_base);
            }
        } else {
#pragma unroll
            for (int e = 0; e < kFlatPer; ++e) {
                const int32_t i = b0 + e;
                unsigned long long c = 3u;
                if (i < tile.end) {
                    if (a.cls) {
                        c = a.cls[i];
                    } else {
                        const int32_t sv = state[i];
                        c = sv == ci ? 1u : sv == cs ? 0u : sv == cr ? 2u : 3u;
                    }
                }
                cw = (cw & ~(0xFFull << (8 * e))) | (c << (8 * e));
                k[e] = c == 0u ? a.cnt[i] : 0;
                l[e] = c <= 1u ? (lids ? __ldg(lids + i) : (uint32_t)(i - lid_base)) : 0u;
            }
        }
        // 2. draws per agent: a recovery draw per infected agent, min(k, kFlatCap)
        //    infection draws (SIR-A: one) per susceptible agent with k > 0 (the
        //    class bytes compared four at a time: a byte equal to 0 or 1 becomes
        //    0xFF, and the bytes' low bits are gathered into a mask)
        const uint32_t cl_lo = (uint32_t)cw, cl_hi = (uint32_t)(cw >> 32);
        const uint32_t smask = class_mask4(cl_lo, 0u) | (class_mask4(cl_hi, 0u) << 4);
        const uint32_t imask = class_mask4(cl_lo, 1u) | (class_mask4(cl_hi, 1u) << 4);
        uint32_t cand = imask, more = 0;
        int32_t ndraw = __popc(imask);
#pragma unroll
        for (int e = 0; e < kFlatPer; ++e) {
            k[e] = (smask >> e) & 1u ? k[e] : 0;
            cand |= (uint32_t)(k[e] > 0) << e;
            ndraw += VARIANT == 1 ? (k[e] > 0) : min(k[e], kFlatCap);
            if (VARIANT == 2) more |= (uint32_t)(k[e] > kFlatCap) << e;
        }
        // 3. warp scan of (candidates << 32 | draws); this lane's candidates go
        //    to the warp's lists
        const unsigned long long mine = ((unsigned long long)__popc(cand) << 32) | (unsigned)ndraw;
        unsigned long long x = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        const unsigned long long wtot = __shfl_sync(FULL_MASK, x, 31);
        const int32_t ncand = (int32_t)(wtot >> 32), ntot = (int32_t)(wtot & 0xFFFFFFFFull);
        {
            const unsigned long long ex = x - mine;
            int32_t cpos = (int32_t)(ex >> 32), dpos = (int32_t)(ex & 0xFFFFFFFFull);
#pragma unroll
            for (int e = 0; e < kFlatPer; ++e)
                if ((cand >> e) & 1u) {
                    const bool rec = (imask >> e) & 1u;
                    const int32_t dn = dpos + (rec || VARIANT == 1 ? 1 : min(k[e], kFlatCap));
                    // Philox counter of draw d is base + d: salt 1 for a recovery
                    // (and SIR-A), salt 2 + j for the j-th SIR-B draw
                    sh_rec[warp][cpos] = make_uint4(c0b + (rec || VARIANT == 1 ? 1u : 2u) - (uint32_t)dpos, l[e],
                                                    rec ? krec : kinf,
                                                    (uint32_t)dn | ((uint32_t)(lane * kFlatPer + e) << 16));
                    ++cpos;
                    dpos = dn;
                }
        }
        if (lane < kFlatWarpAgents / 32) sh_hit[warp][lane] = 0u;
        __syncwarp();
        // 4. an equal share of the warp's draws per lane, kFlatIlp side by side
        {
            const int32_t per = (ntot + 31) >> 5;
            int32_t d = lane * per;
            const int32_t dend = min(d + per, ntot);
            if (d < dend) {
                const uint4 *recs = sh_rec[warp];
                int32_t lo = 0, hi = ncand - 1; // owner of draw d: the first c whose draws end after d
                while (lo < hi) {
                    const int32_t mid = (lo + hi) >> 1;
                    if ((int32_t)(recs[mid].w & 0xFFFFu) > d) hi = mid;
                    else lo = mid + 1;
                }
                int32_t c = lo;
                uint4 cr4 = recs[c]; // counter base, RNG key, threshold, end of draws | agent << 16
                // every candidate has at least one draw, so consecutive draws
                // belong to the same candidate or to the next one
                auto next = [&](int32_t dd) {
                    if (dd >= (int32_t)(cr4.w & 0xFFFFu)) cr4 = recs[++c];
                };
                for (; d + kFlatIlp <= dend; d += kFlatIlp) {
                    uint32_t c0[kFlatIlp], c1[kFlatIlp], th[kFlatIlp], in[kFlatIlp];
#pragma unroll
                    for (int u = 0; u < kFlatIlp; ++u) {
                        next(d + u);
                        c0[u] = cr4.x + (uint32_t)(d + u);
                        c1[u] = cr4.y;
                        th[u] = cr4.z;
                        in[u] = cr4.w >> 16;
                    }
                    philox_k23_ilp<kFlatIlp>(c0, c1, ks);
#pragma unroll
                    for (int u = 0; u < kFlatIlp; ++u)
                        if (c0[u] < th[u]) atomicOr(&sh_hit[warp][in[u] >> 5], 1u << (in[u] & 31u));
                }
                for (; d < dend; ++d) { // the last few, one at a time
                    next(d);
                    if (sg_philox_k23_keys(cr4.x + (uint32_t)d, cr4.y, ks) < cr4.z)
                        atomicOr(&sh_hit[warp][(cr4.w >> 16) >> 5], 1u << ((cr4.w >> 16) & 31u));
                }
            }
        }
        __syncwarp();
        uint32_t hits = (sh_hit[warp][lane >> 2] >> ((lane & 3) * kFlatPer)) & 0xFFu;
        // 5. draws kFlatCap .. k-1 of susceptible agents that need more, warp-wide
        if (VARIANT == 2 && __any_sync(FULL_MASK, more & ~hits)) {
#pragma unroll
            for (int e = 0; e < kFlatPer; ++e) {
                unsigned m = __ballot_sync(FULL_MASK, ((more & ~hits) >> e) & 1u);
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    const int32_t bk = __shfl_sync(FULL_MASK, k[e], src);
                    const uint32_t bl = __shfl_sync(FULL_MASK, l[e], src);
                    const bool h = warp_draws((uint32_t)kFlatCap, bk - kFlatCap, c0b, bl, key, kinf, lane);
                    if (lane == src && h) hits |= 1u << e;
                }
            }
        }
        // 6. transitions: the warp's changed agents are listed in shared memory
        //    (the candidate records are no longer read), then each lane applies
        //    every 32nd: state in place, class byte, change-list entry and row.
        //    Changes are sparse, so this runs one or two rounds instead of a
        //    pass over each lane's 8 agents.
        int32_t nw = 0;
        if (__any_sync(FULL_MASK, hits)) {
            const int32_t nh = __popc(hits);
            int32_t incl = nh;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(FULL_MASK, incl, o);
                if (lane >= o) incl += y;
            }
            nw = __shfl_sync(FULL_MASK, incl, 31);
            // agent in the warp's 256 | 0x100 for a recovery (over the candidate records)
            uint16_t *const hl = reinterpret_cast<uint16_t *>(sh_rec[warp]);
            int32_t pos = incl - nh;
#pragma unroll
            for (int e = 0; e < kFlatPer; ++e)
                if ((hits >> e) & 1u) hl[pos++] = (uint16_t)((lane * kFlatPer + e) | (((imask >> e) & 1u) << 8));
            __syncwarp();
            for (int32_t q = lane; q < nw; q += 32) {
                const uint32_t h = hl[q];
                const int32_t i = wfirst + (int32_t)(h & 0xFFu);
                const bool rec = (h >> 8) != 0;
                state[i] = rec ? cr : ci;
                if (a.cls) a.cls[i] = (uint8_t)(rec ? 2 : 1);
                a.changes[wfirst + q] = rec ? ~i : i;
                record_changed_row(a, wfirst + q, i, rec ? -1 : 1);
            }
        }
        if (STATS) {
            unsigned long long nS = 0, nI = 0, nR = 0, eS = 0;
#pragma unroll
            for (int e = 0; e < kFlatPer; ++e) {
                const int32_t i = b0 + e;
                const uint32_t c = (uint32_t)(cw >> (8 * e)) & 0xFFu;
                if (c == 0u) eS += (unsigned long long)(__ldg(a.off + i + 1) - __ldg(a.off + i));
                const uint32_t after = (hits >> e) & 1u ? ((imask >> e) & 1u ? 2u : 1u) : c;
                nS += after == 0u;
                nI += after == 1u;
                nR += after == 2u;
            }
            if (a.segs[tile.seg].stats)
                block_flush4(nS, nI, nR, eS, a.segs[tile.seg].stats + 4 * (int64_t)a.r, red);
        }
        // 7. the tile's change count, and each warp's changes as chunks of at
        //    most 32 on the scatter's work list (one list allocation per tile)
        if (lane == 0) sh_nw[warp] = nw;
        __syncthreads();
        if (warp == 0) {
            const int32_t n = lane < kWarps ? sh_nw[lane] : 0;
            const int32_t ck = (n + 31) >> 5;
            int32_t cin = ck, nin = n;
#pragma unroll
            for (int o = 1; o < kWarps; o <<= 1) {
                const int32_t y = __shfl_up_sync(FULL_MASK, cin, o);
                const int32_t z = __shfl_up_sync(FULL_MASK, nin, o);
                if (lane >= o) {
                    cin += y;
                    nin += z;
                }
            }
            if (lane < kWarps) sh_coff[lane] = cin - ck;
            const int32_t ctot = __shfl_sync(FULL_MASK, cin, kWarps - 1);
            const int32_t ntile = __shfl_sync(FULL_MASK, nin, kWarps - 1);
            if (lane == 0) {
                a.tile_nch[t] = ntile;
                if (a.tick_changes && ntile > 0) atomicAdd(a.tick_changes + a.r, ntile);
                if (a.tick_cand) atomicAdd(a.tick_cand + a.r, tile.end - tile.begin);
                sh_cbase = ctot > 0 ? atomicAdd(a.nchunks + a.r, ctot) : 0;
            }
        }
        __syncthreads();
        if (nw > 0) {
            const int32_t base = sh_cbase + sh_coff[warp];
            for (int32_t j = lane; j < ((nw + 31) >> 5); j += 32)
                a.chunks[base + j] = SgChunk{wfirst + 32 * j, min(32, nw - 32 * j)};
        }
    }
}

template <int VARIANT, bool STATS>
__global__ void __launch_bounds__(SG_SIR_THREADS, kFlatBlocksPerSm) sir_count_flat_kernel(SgTickArgs a)
{
    __shared__ SgFlatSmem sm;
    if (a.hybrid_rise > 0 && !hybrid_loop_tick(a)) return; // the class sweep takes this tick
    flat_tick<VARIANT, STATS>(a, sm);
}
