// sg_batch.h -- the scenario pool shared by the ensemble batch and the server.
//
// A pool holds many independent SIR scenarios in one set of device arrays:
//   agent slots  [agent_base, agent_base + n + 1): the extra slot keeps each
//                scenario's offsets self-contained (off[agent_base + n] is the
//                end of its last row), so scenarios can come and go;
//   edge slots   [edge_base, edge_base + nnz): CSR entries as global indices;
//   state        int32 per agent slot (updated in place by the count strategy;
//                the pull strategy ping-pongs with a second buffer);
//   cnt/changes  count-strategy scratch per agent slot, with the class byte the
//                class sweep reads;
//   segs         one SgSeg per scenario (tick counter, horizon, seed, codes);
//   tiles        the work list of the kernels, tiles never straddle scenarios.
// Space is handed out first-fit from free lists of agent and edge slots.
#pragma once
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sg_internal.h"

// Agent slots of a scenario of n agents: n + 1, rounded up to a multiple of 32
// (128-bit loads, and class-sweep mask words that belong to one scenario).
inline int64_t sg_pool_agent_slots(int64_t n) { return (n + 1 + 31) & ~int64_t(31); }

// Host threads that split a job (a memcpy, a scan) among themselves and the
// caller; started once and kept (a thread start per piece of work costs more
// than copying a few MB).
class SgCopyWorkers {
  public:
    explicit SgCopyWorkers(unsigned n)
    {
        for (unsigned i = 0; i < n; ++i) th_.emplace_back([this] { run(); });
    }
    ~SgCopyWorkers()
    {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        wake_.notify_all();
        for (auto &t : th_) t.join();
    }
    SgCopyWorkers(const SgCopyWorkers &) = delete;
    SgCopyWorkers &operator=(const SgCopyWorkers &) = delete;

    unsigned threads() const { return (unsigned)th_.size() + 1; }

    // Runs job(0) .. job(parts - 1) on the workers and the caller; returns when
    // all have finished.
    void run_parts(unsigned parts, std::function<void(unsigned)> job)
    {
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = std::move(job);
            parts_ = parts;
            next_ = 0;
            left_ = parts;
            ++gen_;
        }
        wake_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [this] { return left_ == 0; });
    }

    // dst[0, len) = src[0, len), one part per thread.
    void copy(char *dst, const char *src, size_t len)
    {
        const unsigned parts = threads();
        const size_t part = ((len + parts - 1) / parts + 63) & ~(size_t)63;
        run_parts(parts, [=](unsigned k) {
            const size_t b = (size_t)k * part;
            if (b < len) memcpy(dst + b, src + b, std::min(part, len - b));
        });
    }

  private:
    void work()
    {
        for (;;) {
            unsigned k;
            {
                std::lock_guard<std::mutex> g(m_);
                if (next_ >= parts_) return;
                k = next_++;
            }
            job_(k);
            std::lock_guard<std::mutex> g(m_);
            if (--left_ == 0) done_.notify_all();
        }
    }
    void run()
    {
        unsigned long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                wake_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable wake_, done_;
    std::function<void(unsigned)> job_;
    unsigned parts_ = 0, next_ = 0, left_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false;
};

struct SgPoolScen {
    int32_t sid = -1;
    int64_t n = 0, nnz = 0;
    int64_t agent_base = -1, edge_base = -1;
    int64_t tick = 0;     // ticks done
    int64_t horizon = 0;  // ticks to do
    int32_t par = 0;      // state lives in buffer [par] (pull ping-pong)
    bool cnt_valid = false;
    sg_scenario_desc d{}; // host pointers are not kept
    uint32_t key = 0, kinf = 0, krec = 0;
    std::vector<uint32_t> lids; // empty: lid = local index
    bool has_lids = false;      // keys in the pool's logical-id array (else the local index)
    bool symmetric = true;
};

// Free-list allocator over [0, cap) (first fit, coalescing on release).
struct SgRanges {
    int64_t cap = 0;
    std::map<int64_t, int64_t> free_; // start -> length
    void reset(int64_t c)
    {
        cap = c;
        free_.clear();
        if (c > 0) free_[0] = c;
    }
    int64_t take(int64_t len);
    void give(int64_t start, int64_t len);
    int64_t largest() const;
};

struct SgPool {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 152;
    std::string err;

    int64_t agent_cap = 0, edge_cap = 0;
    SgRanges agents, edges;
    SgDev off, idx, toff, tidx, st[2], cnt, changes, tile_nch, lids, segs, tiles, mega, chunks, nchunks,
        rowsegs, nrowsegs, cls, amask, mrebuild, tick_changes;
    int32_t nchunks_cap = 0;
    SgDev snap_st[2], snap_cnt, snap_cls;
    SgDev check_flag; // int32 result of sg_launch_check_csr
    // Large host -> device uploads go through two pinned staging buffers that
    // several host threads fill while the other one is in flight; a copy from
    // pageable memory runs far below the link's bandwidth.
    void *stage[2] = {nullptr, nullptr};
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    std::unique_ptr<SgCopyWorkers> copiers; // started with the staging buffers
    int upload(void *dst, const void *src, size_t bytes);
    SgCopyWorkers &workers(); // started on first use
    bool any_lids = false, all_symmetric = true;
    int64_t seg_cap = 0, tile_cap = 0, mega_cap = 0;

    std::vector<SgPoolScen> scen; // by slot; sid -> slot via sid_slot
    std::map<int32_t, size_t> sid_slot;
    int32_t next_sid = 0;
    int32_t builtin = 0; // SIR variant shared by the pool

    std::vector<SgSeg> hsegs;
    std::vector<SgTile> htiles;
    std::vector<SgMega> hmega;
    bool tables_dirty = true;
    uint64_t version = 1;

    sg_tune tune{SG_SIR_COUNT, 16, 32, 2048, SG_FLAVOUR_SWEEP | SG_FLAVOUR_HYBRID, 0.0};
    cudaGraphExec_t graph = nullptr;
    int32_t graph_nticks = -1;
    uint64_t graph_version = 0;
    sg_tune graph_tune{};

    int fail(int code, const std::string &m)
    {
        err = m;
        return code;
    }
    int cuda_fail(cudaError_t ce, const char *what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(ce);
        return ce == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }

    int init(const sg_engine_cfg *cfg);
    void destroy();
    // Device arrays for the given capacities (contents of a smaller pool are
    // not kept: call before placing scenarios).
    int allocate(int64_t agent_cap, int64_t edge_cap, int64_t max_scen, bool transpose, bool lids);
    // Places one scenario (uploads CSR, state, lids). check_on_device: the CSR
    // has not been checked on the host; its offsets must start at 0 and end at
    // nnz, and the rest (monotone offsets, indices in range) is checked on the
    // device before anything is kept (SG_ERR_BAD_CSR, nothing placed).
    int place(const sg_scenario_desc &d, const int32_t *off, const int32_t *idx, const int32_t *state,
              const int64_t *lids, int32_t sid, bool check_on_device = false);
    void release(int32_t sid);
    bool fits(int64_t n, int64_t nnz) const;
    int rebuild_tables();
    // Enqueues nticks ticks (and the count-strategy init where needed).
    int run(int32_t nticks, bool use_graph);
    int snapshot();
    int restore();
    int get_state(int32_t sid, int32_t *host, int64_t n);
    int consolidate(); // moves every scenario's state to buffer 0
    size_t device_bytes() const;

    // scenario id -> its rows longer than the smallest tunable mega_row
    // (local agent, length)
    std::map<int32_t, std::vector<std::pair<int32_t, int32_t>>> s_long_rows_;
    struct SnapHost {
        int64_t tick;
        int32_t par;
        bool cnt_valid;
    };
    std::vector<SnapHost> snap_host_;

  private:
    int enqueue(int32_t nticks, bool capturing);
    int upload_segs();
};

// bytes of device memory a scenario of n agents and nnz entries occupies
int64_t sg_pool_scenario_bytes(int64_t n, int64_t nnz, bool transpose, bool lids);
