// sg_batch.cu -- scenario pool and the ensemble batch C ABI.
//
// An ensemble of independent SIR scenarios with uneven sizes runs as one
// problem: every scenario is a segment of one device pool and every kernel
// launch walks the tiles of all of them, so a 1,000-agent scenario costs its
// share of one launch instead of a launch of its own. Per-scenario tick
// counters live in the segment table, which the kernels read; a captured CUDA
// graph of the tick loop therefore serves every run of the same length.
#include <algorithm>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>

#include "sg_batch.h"
#include "sg_philox.h"

#define POOL_CK(call)                                                                          \
    do {                                                                                       \
        cudaError_t _ce = (call);                                                              \
        if (_ce != cudaSuccess) return cuda_fail(_ce, #call);                                  \
    } while (0)

void sg_set_thread_error(const std::string &msg); // sg_engine.cu

namespace {
constexpr int32_t kLongRowFloor = 512; // rows kept as mega candidates (smallest tunable mega_row)
// count-step flavours the autotuner times: loop form (4 or 8 agents per thread,
// eager or lazy loads, per-lane or warp-dense draws) and class sweep with the
// load-balanced scatter (alone or in the hybrid), two of them with the
// lane-per-row scatter, and flat draws (every tick, or the hybrid's busy ticks)
constexpr int32_t kCountFlavourCands[] = {0,
                                          1,
                                          4,
                                          5,
                                          SG_FLAVOUR_DENSE,
                                          SG_FLAVOUR_DENSE | SG_FLAVOUR_LAZY,
                                          SG_FLAVOUR_SWEEP | SG_FLAVOUR_HYBRID | SG_FLAVOUR_DENSE | SG_FLAVOUR_LAZY,
                                          SG_FLAVOUR_SWEEP,
                                          SG_FLAVOUR_SWEEP | SG_FLAVOUR_FORCE,
                                          SG_FLAVOUR_SWEEP | SG_FLAVOUR_HYBRID,
                                          SG_FLAVOUR_SWEEP | SG_FLAVOUR_FORCE | SG_FLAVOUR_HYBRID,
                                          SG_FLAVOUR_ROWSCATTER | 4,
                                          SG_FLAVOUR_ROWSCATTER | SG_FLAVOUR_SWEEP,
                                          SG_FLAVOUR_FLAT | 4,
                                          SG_FLAVOUR_SWEEP | SG_FLAVOUR_HYBRID | SG_FLAVOUR_FLAT | SG_FLAVOUR_DENSE |
                                              SG_FLAVOUR_LAZY};
}

int64_t SgRanges::take(int64_t len)
{
    if (len <= 0) len = 1;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= len) {
            const int64_t start = it->first, rest = it->second - len;
            free_.erase(it);
            if (rest > 0) free_[start + len] = rest;
            return start;
        }
    }
    return -1;
}

void SgRanges::give(int64_t start, int64_t len)
{
    if (len <= 0) len = 1;
    auto it = free_.emplace(start, len).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}

int64_t SgRanges::largest() const
{
    int64_t m = 0;
    for (auto &kv : free_) m = std::max(m, kv.second);
    return m;
}

int64_t sg_pool_scenario_bytes(int64_t n, int64_t nnz, bool transpose, bool lids)
{
    const int64_t per_agent = 4 /*off*/ + 8 /*state x2*/ + 8 /*cnt, changes*/ + 2 /*class, activity bit*/ +
                              (lids ? 4 : 0) + (transpose ? 4 : 0);
    const int64_t per_edge = 4 + (transpose ? 4 : 0);
    const int64_t tiles = (n + SG_TILE - 1) / SG_TILE + 1;
    const int64_t rowseg_bytes = (int64_t)SG_ROWSEG_CAPACITY(nnz) * (int64_t)sizeof(SgRowSeg); // the scatter's segment list
    return sg_pool_agent_slots(n) * per_agent + nnz * per_edge + rowseg_bytes + tiles * (int64_t)(sizeof(SgTile) + 4) +
           (int64_t)sizeof(SgSeg);
}

int SgPool::init(const sg_engine_cfg *cfg)
{
    device = cfg ? cfg->device : 0;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev <= 0) return fail(SG_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    if (device < 0 || device >= ndev) return fail(SG_ERR_INVALID, "device ordinal out of range");
    POOL_CK(cudaSetDevice(device));
    sm_count = sg_sm_count(device);
    if (cfg && cfg->stream) {
        stream = (cudaStream_t)cfg->stream;
    } else {
        POOL_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    return SG_OK;
}

void SgPool::destroy()
{
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    copiers.reset();
    for (int h = 0; h < 2; ++h) {
        if (stage[h]) cudaFreeHost(stage[h]);
        if (stage_ev[h]) cudaEventDestroy(stage_ev[h]);
        stage[h] = nullptr;
        stage_ev[h] = nullptr;
    }
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    if (own_stream && stream) cudaStreamDestroy(stream);
    stream = nullptr;
}

namespace {
constexpr size_t kStageBytes = (size_t)32 << 20;
constexpr size_t kStageMin = (size_t)4 << 20; // smaller uploads: one direct copy

} // namespace

SgCopyWorkers &SgPool::workers()
{
    if (!copiers) {
        const unsigned hc = std::thread::hardware_concurrency();
        copiers.reset(new SgCopyWorkers(hc > 1 ? std::min(7u, hc - 1) : 0u));
    }
    return *copiers;
}

int SgPool::upload(void *dst, const void *src, size_t bytes)
{
    if (bytes < kStageMin) {
        POOL_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
        return SG_OK;
    }
    {
        // page-locked source (e.g. a server's receive buffers): one direct copy
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, src) == cudaSuccess && at.type == cudaMemoryTypeHost) {
            POOL_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
            return SG_OK;
        }
        (void)cudaGetLastError();
    }
    if (!stage[0]) {
        for (int h = 0; h < 2; ++h) {
            POOL_CK(cudaHostAlloc(&stage[h], kStageBytes, cudaHostAllocDefault));
            POOL_CK(cudaEventCreateWithFlags(&stage_ev[h], cudaEventDisableTiming));
        }
    }
    SgCopyWorkers &cw = workers();
    int h = 0;
    for (size_t pos = 0; pos < bytes; pos += kStageBytes, h ^= 1) {
        const size_t len = std::min(kStageBytes, bytes - pos);
        POOL_CK(cudaEventSynchronize(stage_ev[h])); // this buffer's previous copy has left
        cw.copy((char *)stage[h], (const char *)src + pos, len);
        POOL_CK(cudaMemcpyAsync((char *)dst + pos, stage[h], len, cudaMemcpyHostToDevice, stream));
        POOL_CK(cudaEventRecord(stage_ev[h], stream));
    }
    return SG_OK;
}

int SgPool::allocate(int64_t acap, int64_t ecap, int64_t max_scen, bool transpose, bool with_lids)
{
    POOL_CK(cudaSetDevice(device));
    agent_cap = acap;
    edge_cap = ecap;
    seg_cap = std::max<int64_t>(max_scen, 1);
    tile_cap = acap / SG_TILE + seg_cap + 1;
    POOL_CK(off.reserve((size_t)(acap + 1) * 4));
    POOL_CK(idx.reserve((size_t)std::max<int64_t>(ecap, 1) * 4));
    if (transpose) {
        POOL_CK(toff.reserve((size_t)(acap + 1) * 4));
        POOL_CK(tidx.reserve((size_t)std::max<int64_t>(ecap, 1) * 4));
    }
    all_symmetric = !transpose;
    for (auto &b : st) POOL_CK(b.reserve((size_t)std::max<int64_t>(acap, 1) * 4));
    POOL_CK(cnt.reserve((size_t)std::max<int64_t>(acap, 1) * 4));
    POOL_CK(cls.reserve(((size_t)acap + 16) & ~size_t(15)));
    POOL_CK(amask.reserve(((size_t)acap / 32 + 2) * 4));
    POOL_CK(changes.reserve((size_t)std::max<int64_t>(acap, 1) * 4));
    POOL_CK(tile_nch.reserve((size_t)tile_cap * 4));
    POOL_CK(chunks.reserve(((size_t)acap / 32 + (size_t)tile_cap + 1) * sizeof(SgChunk)));
    POOL_CK(rowsegs.reserve(SG_ROWSEG_CAPACITY(ecap) * sizeof(SgRowSeg)));
    POOL_CK(tiles.reserve((size_t)tile_cap * sizeof(SgTile)));
    POOL_CK(segs.reserve((size_t)seg_cap * sizeof(SgSeg)));
    any_lids = with_lids;
    if (with_lids) POOL_CK(lids.reserve((size_t)std::max<int64_t>(acap, 1) * 4));
    agents.reset(acap);
    edges.reset(ecap);
    return SG_OK;
}

bool SgPool::fits(int64_t n, int64_t nnz) const
{
    return agents.largest() >= sg_pool_agent_slots(n) && (nnz == 0 || edges.largest() >= nnz) &&
           (int64_t)scen.size() < seg_cap;
}

int SgPool::place(const sg_scenario_desc &d, const int32_t *loff, const int32_t *lidx, const int32_t *state,
                  const int64_t *llids, int32_t sid, bool check_on_device)
{
    const int64_t n = d.n_agents, nnz = d.nnz;
    if (builtin == 0) builtin = d.builtin;
    if (d.builtin != builtin) return fail(SG_ERR_INVALID, "all scenarios of a pool use the same SIR builtin");
    const bool sym = (d.flags & SG_GRAPH_SYMMETRIC) != 0;
    if (!sym && all_symmetric) return fail(SG_ERR_INVALID, "pool holds symmetric graphs only");
    if (llids && !any_lids) return fail(SG_ERR_INVALID, "pool was allocated without logical ids");
    if ((int64_t)scen.size() >= seg_cap) return fail(SG_ERR_BUDGET, "scenario table full");
    const int64_t aslots = sg_pool_agent_slots(n);
    const int64_t ab = agents.take(aslots);
    if (ab < 0) return fail(SG_ERR_BUDGET, "no room for the scenario's agents");
    const int64_t eb = nnz > 0 ? edges.take(nnz) : 0;
    if (eb < 0) {
        agents.give(ab, aslots);
        return fail(SG_ERR_BUDGET, "no room for the scenario's edges");
    }
    POOL_CK(cudaSetDevice(device));
    // local CSR copied as is, then shifted to pool slots on the device
    int urc = upload(off.as<int32_t>() + ab, loff, (size_t)(n + 1) * 4);
    if (!urc && nnz) urc = upload(idx.as<int32_t>() + eb, lidx, (size_t)nnz * 4);
    if (urc) {
        agents.give(ab, aslots);
        if (nnz) edges.give(eb, nnz);
        return urc;
    }
    if (check_on_device) {
        int32_t bad = 0;
        POOL_CK(check_flag.reserve(4));
        POOL_CK(cudaMemsetAsync(check_flag.p, 0, 4, stream));
        POOL_CK(sg_launch_check_csr(off.as<int32_t>() + ab, n, idx.as<int32_t>() + eb, nnz, check_flag.as<int32_t>(),
                                    stream));
        POOL_CK(cudaMemcpyAsync(&bad, check_flag.p, 4, cudaMemcpyDeviceToHost, stream));
        POOL_CK(cudaStreamSynchronize(stream));
        if (bad) {
            agents.give(ab, aslots);
            if (nnz) edges.give(eb, nnz);
            return fail(SG_ERR_BAD_CSR, bad == 1 ? "offsets decrease" : "an index is outside [0, n)");
        }
    }
    POOL_CK(sg_launch_offset_csr(off.as<int32_t>() + ab, n + 1, (int32_t)eb, idx.as<int32_t>() + eb, nnz,
                                 (int32_t)ab, stream));
    if (!all_symmetric) {
        // transpose rows (in-neighbours) of this scenario, placed in the same slots
        std::vector<int32_t> tcount((size_t)n + 1, 0), tcur((size_t)n);
        for (int64_t k = 0; k < nnz; ++k) tcount[(size_t)lidx[k] + 1]++;
        for (int64_t i = 0; i < n; ++i) tcount[(size_t)i + 1] += tcount[(size_t)i];
        for (int64_t i = 0; i < n; ++i) tcur[(size_t)i] = tcount[(size_t)i];
        std::vector<int32_t> t((size_t)nnz);
        for (int64_t i = 0; i < n; ++i)
            for (int32_t k = loff[i]; k < loff[i + 1]; ++k) t[(size_t)tcur[(size_t)lidx[k]]++] = (int32_t)(ab + i);
        for (int64_t i = 0; i <= n; ++i) tcount[(size_t)i] += (int32_t)eb;
        POOL_CK(cudaMemcpyAsync(toff.as<int32_t>() + ab, tcount.data(), (size_t)(n + 1) * 4, cudaMemcpyHostToDevice, stream));
        if (nnz) POOL_CK(cudaMemcpyAsync(tidx.as<int32_t>() + eb, t.data(), (size_t)nnz * 4, cudaMemcpyHostToDevice, stream));
    }
    {
        const int rc = upload(st[0].as<int32_t>() + ab, state, (size_t)n * 4);
        if (rc) {
            agents.give(ab, aslots);
            if (nnz) edges.give(eb, nnz);
            return rc;
        }
    }
    SgPoolScen s;
    s.sid = sid;
    s.n = n;
    s.nnz = nnz;
    s.agent_base = ab;
    s.edge_base = eb;
    s.tick = 0;
    s.horizon = d.horizon;
    s.par = 0;
    s.cnt_valid = false;
    s.d = d;
    s.d.offsets = s.d.indices = s.d.state = nullptr;
    s.d.lids = nullptr;
    s.key = (uint32_t)(uint64_t)d.seed;
    s.kinf = sg_threshold_host(d.beta);
    s.krec = sg_threshold_host(d.gamma);
    s.symmetric = sym;
    // a scenario without logical ids keys its draws on the local index, which
    // the kernels derive from the segment's base (its segment has no lids)
    s.has_lids = llids != nullptr;
    if (llids) {
        std::vector<uint32_t> k((size_t)n);
        for (int64_t i = 0; i < n; ++i) k[(size_t)i] = (uint32_t)(uint64_t)llids[i];
        POOL_CK(cudaMemcpyAsync(lids.as<uint32_t>() + ab, k.data(), (size_t)n * 4, cudaMemcpyHostToDevice, stream));
    }
    // long rows (candidates for whole-block scans), in index order; large
    // scenarios scan their offsets on the worker threads
    std::vector<std::pair<int32_t, int32_t>> longs;
    auto scan_rows = [loff](int64_t b, int64_t e, std::vector<std::pair<int32_t, int32_t>> &out) {
        for (int64_t i = b; i < e; ++i)
            if (loff[i + 1] - loff[i] > kLongRowFloor) out.push_back({(int32_t)i, loff[i + 1] - loff[i]});
    };
    if (n < ((int64_t)1 << 20)) {
        scan_rows(0, n, longs);
    } else {
        SgCopyWorkers &cw = workers();
        const unsigned parts = cw.threads();
        const int64_t step = (n + parts - 1) / parts;
        std::vector<std::vector<std::pair<int32_t, int32_t>>> found(parts);
        cw.run_parts(parts, [&](unsigned k) {
            scan_rows(std::min(n, (int64_t)k * step), std::min(n, (int64_t)(k + 1) * step), found[k]);
        });
        for (auto &f : found) longs.insert(longs.end(), f.begin(), f.end());
    }
    POOL_CK(cudaStreamSynchronize(stream)); // host staging vectors go out of scope
    s_long_rows_[sid] = std::move(longs);
    sid_slot[sid] = scen.size();
    scen.push_back(std::move(s));
    tables_dirty = true;
    version++;
    return SG_OK;
}

void SgPool::release(int32_t sid)
{
    auto it = sid_slot.find(sid);
    if (it == sid_slot.end()) return;
    const size_t slot = it->second;
    agents.give(scen[slot].agent_base, sg_pool_agent_slots(scen[slot].n));
    if (scen[slot].nnz) edges.give(scen[slot].edge_base, scen[slot].nnz);
    s_long_rows_.erase(sid);
    scen.erase(scen.begin() + (ptrdiff_t)slot);
    sid_slot.clear();
    for (size_t i = 0; i < scen.size(); ++i) sid_slot[scen[i].sid] = i;
    tables_dirty = true;
    version++;
}

int SgPool::rebuild_tables()
{
    htiles.clear();
    hmega.clear();
    for (size_t k = 0; k < scen.size(); ++k) {
        const SgPoolScen &s = scen[k];
        sg_append_tiles(htiles, (int32_t)k, s.agent_base, s.agent_base + s.n);
        auto lr = s_long_rows_.find(s.sid);
        if (lr != s_long_rows_.end())
            for (auto &p : lr->second)
                if (p.second > tune.mega_row) hmega.push_back(SgMega{(int32_t)(s.agent_base + p.first), (int32_t)k});
    }
    if ((int64_t)htiles.size() > tile_cap) return fail(SG_ERR_INVALID, "tile table overflow");
    if (!htiles.empty())
        POOL_CK(cudaMemcpyAsync(tiles.p, htiles.data(), htiles.size() * sizeof(SgTile), cudaMemcpyHostToDevice, stream));
    POOL_CK(mega.reserve(std::max<size_t>(hmega.size(), 1) * sizeof(SgMega)));
    if (!hmega.empty())
        POOL_CK(cudaMemcpyAsync(mega.p, hmega.data(), hmega.size() * sizeof(SgMega), cudaMemcpyHostToDevice, stream));
    POOL_CK(cudaStreamSynchronize(stream));
    tables_dirty = false;
    return SG_OK;
}

int SgPool::upload_segs()
{
    hsegs.resize(scen.size());
    for (size_t k = 0; k < scen.size(); ++k) {
        const SgPoolScen &s = scen[k];
        SgSeg &g = hsegs[k];
        memset(&g, 0, sizeof g);
        g.tick0 = s.tick;
        g.end_tick = s.horizon;
        g.lids = any_lids && s.has_lids ? lids.as<uint32_t>() : nullptr;
        g.lid_base = (int32_t)s.agent_base;
        g.variant = builtin;
        g.key = s.key;
        g.kinf = s.kinf;
        g.krec = s.krec;
        g.cs = s.d.code_s;
        g.ci = s.d.code_i;
        g.cr = s.d.code_r;
        g.par0 = s.par;
        g.stats = nullptr;
    }
    if (!hsegs.empty())
        POOL_CK(cudaMemcpyAsync(segs.p, hsegs.data(), hsegs.size() * sizeof(SgSeg), cudaMemcpyHostToDevice, stream));
    return SG_OK;
}

int SgPool::consolidate()
{
    for (auto &s : scen) {
        if (s.par == 0) continue;
        POOL_CK(cudaMemcpyAsync(st[0].as<int32_t>() + s.agent_base, st[1].as<int32_t>() + s.agent_base,
                                (size_t)s.n * 4, cudaMemcpyDeviceToDevice, stream));
        s.par = 0;
    }
    return SG_OK;
}

int SgPool::enqueue(int32_t nticks, bool capturing)
{
    (void)capturing;
    SgTickArgs a{};
    a.off = off.as<int32_t>();
    a.idx = idx.as<int32_t>();
    const bool count = tune.strategy == SG_SIR_COUNT;
    a.buf0 = st[0].p;
    a.buf1 = count ? st[0].p : st[1].p;
    a.segs = segs.as<SgSeg>();
    a.tiles = tiles.as<SgTile>();
    a.ntiles = (int32_t)htiles.size();
    a.thread_row = tune.thread_row;
    a.flavour = tune.count_flavour;
    a.sweep_wpt = sg_sweep_wpt((int64_t)htiles.size(), sm_count, a.flavour);
    sg_hybrid_thresholds((int64_t)htiles.size(), sm_count, a.flavour, &a.hybrid_rise, &a.hybrid_fall);
    if ((a.flavour & SG_FLAVOUR_SWEEP) && !(a.flavour & SG_FLAVOUR_FORCE) &&
        (int64_t)htiles.size() < (int64_t)sm_count * SG_SWEEP_MIN_TILES_PER_SM)
        a.flavour = (a.flavour & ~SG_FLAVOUR_SWEEP) | SG_FLAVOUR_LAZY;
    a.mega = mega.as<SgMega>();
    a.nmega = (int32_t)hmega.size();
    a.mega_blocks = std::min<int32_t>(a.nmega, sm_count);
    a.mega_row = tune.mega_row;
    a.cnt = cnt.as<int32_t>();
    a.changes = changes.as<int32_t>();
    a.tile_nch = tile_nch.as<int32_t>();
    a.chunks = chunks.as<SgChunk>();
    a.nchunks = nchunks.as<int32_t>();
    a.rowsegs = rowsegs.as<SgRowSeg>();
    a.nrowsegs = nrowsegs.as<int32_t>();
    a.toff = all_symmetric ? off.as<int32_t>() : toff.as<int32_t>();
    a.tidx = all_symmetric ? idx.as<int32_t>() : tidx.as<int32_t>();
    if (count) {
        a.cls = cls.as<uint8_t>();
        a.amask = amask.as<uint32_t>();
        a.mrebuild = mrebuild.as<uint8_t>();
        a.tick_changes = tick_changes.as<int32_t>();
    }
    const int grid = std::max(1, std::min<int>(a.ntiles, sm_count * std::max(tune.blocks_per_sm, 1)));
    const int variant = builtin == SG_BUILTIN_SIR_A ? 1 : 2;
    if (a.ntiles == 0) return SG_OK;
    if (count) {
        POOL_CK(cudaMemsetAsync(nchunks.p, 0, (size_t)nticks * 4, stream));
        POOL_CK(cudaMemsetAsync(nrowsegs.p, 0, (size_t)nticks * 4, stream));
        // activity bits are not carried between runs: the first sweep of a run rebuilds them
        POOL_CK(cudaMemsetAsync(mrebuild.p, 0, (size_t)nticks + 1, stream));
        POOL_CK(cudaMemsetAsync(mrebuild.p, 1, 1, stream));
        POOL_CK(cudaMemsetAsync(tick_changes.p, 0, (size_t)nticks * 4, stream));
    }
    for (int32_t r = 0; r < nticks; ++r) {
        a.r = r;
        cudaError_t ce;
        if (count) {
            ce = sg_launch_sir_count_step(a, variant, false, true, grid, stream);
            if (ce == cudaSuccess) ce = sg_launch_sir_count_scatter(a, sm_count * 16, stream);
        } else {
            ce = sg_launch_sir_pull(a, variant, false, grid + a.mega_blocks, stream);
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "tick launch");
    }
    return SG_OK;
}

int SgPool::run(int32_t nticks, bool use_graph)
{
    if (nticks < 0) return fail(SG_ERR_INVALID, "nticks < 0");
    POOL_CK(cudaSetDevice(device));
    if (tables_dirty) {
        int rc = rebuild_tables();
        if (rc) return rc;
    }
    const bool count = tune.strategy == SG_SIR_COUNT;
    if (count && nticks > nchunks_cap) { // before any capture: no allocation inside a graph
        POOL_CK(nchunks.reserve((size_t)nticks * 4));
        POOL_CK(nrowsegs.reserve((size_t)nticks * 4));
        POOL_CK(mrebuild.reserve((size_t)nticks + 1));
        POOL_CK(tick_changes.reserve((size_t)nticks * 4));
        nchunks_cap = nticks;
    }
    if (count) {
        int rc = consolidate();
        if (rc) return rc;
        // counts for scenarios that have none yet (new, or after pull runs)
        std::vector<SgTile> init;
        for (size_t k = 0; k < scen.size(); ++k)
            if (!scen[k].cnt_valid) sg_append_tiles(init, (int32_t)k, scen[k].agent_base, scen[k].agent_base + scen[k].n);
        rc = upload_segs();
        if (rc) return rc;
        if (!init.empty()) {
            SgDev itiles;
            POOL_CK(itiles.reserve(init.size() * sizeof(SgTile)));
            POOL_CK(cudaMemcpyAsync(itiles.p, init.data(), init.size() * sizeof(SgTile), cudaMemcpyHostToDevice, stream));
            SgTickArgs a{};
            a.off = off.as<int32_t>();
            a.idx = idx.as<int32_t>();
            a.buf0 = a.buf1 = st[0].p;
            a.segs = segs.as<SgSeg>();
            a.tiles = itiles.as<SgTile>();
            a.ntiles = (int32_t)init.size();
            a.cnt = cnt.as<int32_t>();
            a.cls = cls.as<uint8_t>();
            a.amask = amask.as<uint32_t>();
            a.mega = nullptr;
            a.nmega = 0;
            a.mega_blocks = 0;
            a.mega_row = std::numeric_limits<int32_t>::max();
            a.thread_row = tune.thread_row;
            const int grid = std::max(1, std::min<int>(a.ntiles, sm_count * 8));
            cudaError_t ce = sg_launch_sir_count_init(a, grid, stream);
            if (ce != cudaSuccess) return cuda_fail(ce, "sir_count_init");
            POOL_CK(cudaStreamSynchronize(stream)); // itiles is freed on return
            for (auto &s : scen) s.cnt_valid = true;
        }
    } else {
        int rc = upload_segs();
        if (rc) return rc;
    }
    if (nticks > 0) {
        if (!use_graph) {
            int rc = enqueue(nticks, false);
            if (rc) return rc;
        } else {
            const bool same_tune = memcmp(&graph_tune, &tune, offsetof(sg_tune, us_per_tick)) == 0;
            if (!graph || graph_nticks != nticks || graph_version != version || !same_tune) {
                if (graph) {
                    cudaGraphExecDestroy(graph);
                    graph = nullptr;
                }
                cudaGraph_t g = nullptr;
                POOL_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                int rc = enqueue(nticks, true);
                cudaError_t ce = cudaStreamEndCapture(stream, &g);
                if (rc) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
                ce = cudaGraphInstantiate(&graph, g, 0);
                cudaGraphDestroy(g);
                if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
                graph_nticks = nticks;
                graph_version = version;
                graph_tune = tune;
            }
            POOL_CK(cudaGraphLaunch(graph, stream));
        }
    }
    for (auto &s : scen) {
        const int64_t adv = std::max<int64_t>(0, std::min<int64_t>(nticks, s.horizon - s.tick));
        s.tick += adv;
        if (!count) {
            s.par ^= (int32_t)(adv & 1);
            s.cnt_valid = false;
        }
    }
    return SG_OK;
}

int SgPool::snapshot()
{
    POOL_CK(cudaSetDevice(device));
    for (int k = 0; k < 2; ++k) {
        POOL_CK(snap_st[k].reserve(st[k].bytes));
        POOL_CK(cudaMemcpyAsync(snap_st[k].p, st[k].p, st[k].bytes, cudaMemcpyDeviceToDevice, stream));
    }
    POOL_CK(snap_cnt.reserve(cnt.bytes));
    POOL_CK(cudaMemcpyAsync(snap_cnt.p, cnt.p, cnt.bytes, cudaMemcpyDeviceToDevice, stream));
    POOL_CK(snap_cls.reserve(cls.bytes));
    POOL_CK(cudaMemcpyAsync(snap_cls.p, cls.p, cls.bytes, cudaMemcpyDeviceToDevice, stream));
    snap_host_.clear();
    for (auto &s : scen) snap_host_.push_back({s.tick, s.par, s.cnt_valid});
    POOL_CK(cudaStreamSynchronize(stream));
    return SG_OK;
}

int SgPool::restore()
{
    if (snap_host_.size() != scen.size()) return fail(SG_ERR_INVALID, "no snapshot of this pool");
    POOL_CK(cudaSetDevice(device));
    for (int k = 0; k < 2; ++k)
        POOL_CK(cudaMemcpyAsync(st[k].p, snap_st[k].p, st[k].bytes, cudaMemcpyDeviceToDevice, stream));
    POOL_CK(cudaMemcpyAsync(cnt.p, snap_cnt.p, cnt.bytes, cudaMemcpyDeviceToDevice, stream));
    POOL_CK(cudaMemcpyAsync(cls.p, snap_cls.p, cls.bytes, cudaMemcpyDeviceToDevice, stream));
    for (size_t k = 0; k < scen.size(); ++k) {
        scen[k].tick = snap_host_[k].tick;
        scen[k].par = snap_host_[k].par;
        scen[k].cnt_valid = snap_host_[k].cnt_valid;
    }
    return SG_OK;
}

int SgPool::get_state(int32_t sid, int32_t *host, int64_t n)
{
    auto it = sid_slot.find(sid);
    if (it == sid_slot.end()) return fail(SG_ERR_NOT_FOUND, "unknown scenario id");
    const SgPoolScen &s = scen[it->second];
    if (n != s.n) return fail(SG_ERR_INVALID, "n differs from the scenario's agent count");
    POOL_CK(cudaSetDevice(device));
    POOL_CK(cudaMemcpyAsync(host, st[s.par].as<int32_t>() + s.agent_base, (size_t)n * 4, cudaMemcpyDeviceToHost, stream));
    POOL_CK(cudaStreamSynchronize(stream));
    return SG_OK;
}

size_t SgPool::device_bytes() const
{
    size_t b = 0;
    for (const SgDev *d : {&off, &idx, &toff, &tidx, &st[0], &st[1], &cnt, &changes, &tile_nch, &lids, &segs,
                           &tiles, &mega, &cls, &amask, &snap_st[0], &snap_st[1], &snap_cnt, &snap_cls})
        b += d->bytes;
    return b;
}

// ---- the batch C ABI ---------------------------------------------------------------

struct SgStaged {
    sg_scenario_desc d;
    std::vector<int32_t> off, idx, state;
    std::vector<int64_t> lids;
    int32_t sid;
};

struct sg_batch {
    SgPool pool;
    std::vector<SgStaged> staged;
    bool committed = false;
    int32_t next_sid = 0;
};

static int check_desc(const sg_scenario_desc *d, std::string *why)
{
    if (!d) {
        *why = "desc is NULL";
        return SG_ERR_INVALID;
    }
    if (d->builtin != SG_BUILTIN_SIR_A && d->builtin != SG_BUILTIN_SIR_B) {
        *why = "builtin must be SG_BUILTIN_SIR_A or SG_BUILTIN_SIR_B";
        return SG_ERR_INVALID;
    }
    if (d->horizon < 0) {
        *why = "horizon < 0";
        return SG_ERR_INVALID;
    }
    if (!d->state && d->n_agents > 0) {
        *why = "state is NULL";
        return SG_ERR_INVALID;
    }
    *why = sg_check_csr(d->offsets, d->n_agents, d->indices, d->nnz);
    return why->empty() ? SG_OK : SG_ERR_BAD_CSR;
}

extern "C" {

int sg_batch_create(const sg_engine_cfg *cfg, sg_batch **out)
{
    if (!out) return SG_ERR_INVALID;
    *out = nullptr;
    auto *b = new sg_batch();
    int rc = b->pool.init(cfg);
    if (rc) {
        sg_set_thread_error(b->pool.err);
        delete b;
        return rc;
    }
    *out = b;
    return SG_OK;
}

int sg_batch_destroy(sg_batch *b)
{
    if (!b) return SG_OK;
    b->pool.destroy();
    delete b;
    return SG_OK;
}

int sg_batch_last_error(const sg_batch *b, char *buf, size_t cap)
{
    if (!buf || !cap) return SG_ERR_INVALID;
    const std::string &m = b ? b->pool.err : std::string();
    const size_t k = std::min(cap - 1, m.size());
    memcpy(buf, m.data(), k);
    buf[k] = '\0';
    return SG_OK;
}

int sg_batch_add_scenario(sg_batch *b, const sg_scenario_desc *d, int32_t *sid)
{
    if (!b || !sid) return SG_ERR_INVALID;
    if (b->committed) return b->pool.fail(SG_ERR_INVALID, "batch already committed");
    std::string why;
    int rc = check_desc(d, &why);
    if (rc) return b->pool.fail(rc, why);
    if (!b->staged.empty() && b->staged[0].d.builtin != d->builtin)
        return b->pool.fail(SG_ERR_INVALID, "all scenarios of a batch use the same SIR builtin");
    SgStaged s;
    s.d = *d;
    s.off.assign(d->offsets, d->offsets + d->n_agents + 1);
    s.idx.assign(d->indices, d->indices + d->nnz);
    s.state.assign(d->state, d->state + d->n_agents);
    if (d->lids) s.lids.assign(d->lids, d->lids + d->n_agents);
    s.sid = b->next_sid++;
    *sid = s.sid;
    b->staged.push_back(std::move(s));
    return SG_OK;
}

int sg_batch_commit(sg_batch *b)
{
    if (!b) return SG_ERR_INVALID;
    if (b->committed) return b->pool.fail(SG_ERR_INVALID, "batch already committed");
    int64_t agents = 0, nnz = 0;
    bool transpose = false, lids = false;
    for (auto &s : b->staged) {
        agents += sg_pool_agent_slots(s.d.n_agents);
        nnz += s.d.nnz;
        transpose |= !(s.d.flags & SG_GRAPH_SYMMETRIC);
        lids |= !s.lids.empty();
    }
    if (agents >= std::numeric_limits<int32_t>::max() || nnz >= std::numeric_limits<int32_t>::max())
        return b->pool.fail(SG_ERR_INVALID, "batch exceeds 2^31 agents or CSR entries");
    int rc = b->pool.allocate(agents, nnz, (int64_t)b->staged.size(), transpose, lids);
    if (rc) return rc;
    for (auto &s : b->staged) {
        rc = b->pool.place(s.d, s.off.data(), s.idx.data(), s.state.data(), s.lids.empty() ? nullptr : s.lids.data(), s.sid);
        if (rc) return rc;
    }
    b->staged.clear();
    b->staged.shrink_to_fit();
    b->committed = true;
    return b->pool.rebuild_tables();
}

int sg_batch_set_tune(sg_batch *b, const sg_tune *t)
{
    if (!b || !t) return SG_ERR_INVALID;
    if (t->strategy != SG_SIR_PULL && t->strategy != SG_SIR_COUNT) return b->pool.fail(SG_ERR_INVALID, "bad strategy");
    if (t->blocks_per_sm < 1 || t->blocks_per_sm > 32 || t->thread_row < 1 || t->mega_row < kLongRowFloor ||
        t->count_flavour < 0 || t->count_flavour > SG_FLAVOUR_MAX)
        return b->pool.fail(SG_ERR_INVALID, "tune parameters out of range");
    const bool mega_changed = t->mega_row != b->pool.tune.mega_row;
    b->pool.tune = *t;
    if (mega_changed) b->pool.tables_dirty = true;
    return SG_OK;
}

int sg_batch_get_tune(sg_batch *b, sg_tune *t)
{
    if (!b || !t) return SG_ERR_INVALID;
    *t = b->pool.tune;
    return SG_OK;
}

int sg_batch_run(sg_batch *b, int32_t nticks, int32_t use_graph)
{
    if (!b) return SG_ERR_INVALID;
    if (!b->committed) return b->pool.fail(SG_ERR_INVALID, "commit the batch before running");
    return b->pool.run(nticks, use_graph != 0);
}

int sg_batch_synchronize(sg_batch *b)
{
    if (!b) return SG_ERR_INVALID;
    cudaSetDevice(b->pool.device);
    cudaError_t ce = cudaStreamSynchronize(b->pool.stream);
    return ce == cudaSuccess ? SG_OK : b->pool.cuda_fail(ce, "cudaStreamSynchronize");
}

int sg_batch_get_state(sg_batch *b, int32_t sid, int32_t *host, int64_t n)
{
    if (!b || !host) return SG_ERR_INVALID;
    return b->pool.get_state(sid, host, n);
}

int sg_batch_scenario_tick(sg_batch *b, int32_t sid, int64_t *tick)
{
    if (!b || !tick) return SG_ERR_INVALID;
    auto it = b->pool.sid_slot.find(sid);
    if (it == b->pool.sid_slot.end()) return b->pool.fail(SG_ERR_NOT_FOUND, "unknown scenario id");
    *tick = b->pool.scen[it->second].tick;
    return SG_OK;
}

int sg_batch_info(sg_batch *b, int64_t *agents, int64_t *nnz, int64_t *device_bytes)
{
    if (!b) return SG_ERR_INVALID;
    int64_t a = 0, e = 0;
    for (auto &s : b->pool.scen) {
        a += s.n;
        e += s.nnz;
    }
    if (agents) *agents = a;
    if (nnz) *nnz = e;
    if (device_bytes) *device_bytes = (int64_t)b->pool.device_bytes();
    return SG_OK;
}

int sg_batch_snapshot(sg_batch *b)
{
    if (!b) return SG_ERR_INVALID;
    return b->pool.snapshot();
}

int sg_batch_restore(sg_batch *b)
{
    if (!b) return SG_ERR_INVALID;
    return b->pool.restore();
}

int sg_batch_tune(sg_batch *b, int32_t ticks, sg_tune *best)
{
    if (!b || ticks < 1) return SG_ERR_INVALID;
    if (!b->committed) return b->pool.fail(SG_ERR_INVALID, "commit the batch before tuning");
    SgPool &p = b->pool;
    int rc = p.snapshot();
    if (rc) return rc;
    const sg_tune orig = p.tune;
    sg_tune win = orig;
    win.us_per_tick = std::numeric_limits<double>::infinity();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // pull: blocks/SM x lane/warp row split x block-row threshold; count:
    // blocks/SM x count-step flavour (its rows matter only once per run)
    std::vector<sg_tune> cands;
    for (int32_t bps : {2, 4, 8, 16}) {
        for (int32_t trow : {16, 32, 64})
            for (int32_t mrow : {1024, 4096}) cands.push_back(sg_tune{SG_SIR_PULL, bps, trow, mrow, 0, 0.0});
        for (int32_t fl : kCountFlavourCands) cands.push_back(sg_tune{SG_SIR_COUNT, bps, 32, 2048, fl, 0.0});
    }
    for (sg_tune t : cands) {
        if ((rc = sg_batch_set_tune(b, &t)) != SG_OK) break;
        if ((rc = p.restore()) != SG_OK) break;
        // untimed pass: count init, table rebuild, caches
        if ((rc = p.run(1, false)) != SG_OK) break;
        if ((rc = p.restore()) != SG_OK) break;
        if (t.strategy == SG_SIR_COUNT && (rc = p.run(0, false)) != SG_OK) break;
        cudaEventRecord(e0, p.stream);
        if ((rc = p.run(ticks, false)) != SG_OK) break;
        cudaEventRecord(e1, p.stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        t.us_per_tick = 1e3 * ms / ticks;
        if (t.us_per_tick < win.us_per_tick) win = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int rc2 = sg_batch_set_tune(b, rc == SG_OK ? &win : &orig);
    int rc3 = p.restore();
    if (rc) return rc;
    if (rc2) return rc2;
    if (rc3) return rc3;
    if (best) *best = win;
    return cudaStreamSynchronize(p.stream) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

} // extern "C"
