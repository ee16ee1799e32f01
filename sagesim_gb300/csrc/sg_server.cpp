// sg_server.cpp -- continuous batching of SIR scenario requests.
//
// A resident scenario pool (sg_batch.h) on one GPU; requests queue on the
// host, are admitted between tick chunks as soon as budget and pool space
// allow, run together with every other resident scenario in one set of
// launches per tick, and leave the pool when they reach their horizon.
#include <algorithm>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <vector>

#include "sg_batch.h"

void sg_set_thread_error(const std::string &msg); // sg_engine.cu

namespace {

struct Request {
    int64_t rid = 0;
    sg_scenario_desc d{};
    std::vector<int32_t> off, idx, state;
    std::vector<int64_t> lids;
    int64_t bytes = 0;
    int32_t status = SG_REQ_QUEUED;
    bool borrowed = false; // d's host pointers are the caller's (SG_REQ_BORROW), no copies
    std::string failure;   // SG_REQ_FAILED: why placement refused it
    int32_t bypassed = 0;
    int64_t tick = 0;
    std::vector<int32_t> result;
};

constexpr int32_t kMaxBypass = 8;

} // namespace

struct sg_server {
    SgPool pool;
    sg_server_cfg cfg{};
    int64_t next_rid = 0;
    int64_t resident_bytes = 0;
    std::deque<int64_t> queue;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    std::map<int64_t, int32_t> rid_sid; // resident requests -> pool scenario id
    int32_t next_sid = 0;
    int64_t ndone = 0;
};

static int admit(sg_server *s)
{
    SgPool &p = s->pool;
    bool blocked = false; // a long-bypassed request reserves the next free space
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        Request &r = *s->reqs[*it];
        const bool budget_ok = s->resident_bytes + r.bytes <= s->cfg.budget_bytes;
        if (!blocked && budget_ok && p.fits(r.d.n_agents, r.d.nnz)) {
            const int32_t sid = s->next_sid++;
            int rc = r.borrowed ? p.place(r.d, r.d.offsets, r.d.indices, r.d.state, r.d.lids, sid, true)
                                : p.place(r.d, r.off.data(), r.idx.data(), r.state.data(),
                                          r.lids.empty() ? nullptr : r.lids.data(), sid);
            if (rc == SG_ERR_BUDGET) { // fragmentation: try later
                ++it;
                continue;
            }
            if (rc == SG_ERR_BAD_CSR && r.borrowed) { // checked on the device only now
                r.status = SG_REQ_FAILED;
                r.failure = p.err;
                r.d.offsets = r.d.indices = r.d.state = nullptr;
                r.d.lids = nullptr;
                it = s->queue.erase(it);
                continue;
            }
            if (rc) return rc;
            r.d.offsets = r.d.indices = r.d.state = nullptr; // the caller's arrays are free again
            r.d.lids = nullptr;
            s->rid_sid[r.rid] = sid;
            s->resident_bytes += r.bytes;
            r.status = SG_REQ_RUNNING;
            std::vector<int32_t>().swap(r.off);
            std::vector<int32_t>().swap(r.idx);
            std::vector<int32_t>().swap(r.state);
            std::vector<int64_t>().swap(r.lids);
            it = s->queue.erase(it);
            continue;
        }
        if (++r.bypassed >= kMaxBypass) blocked = true;
        ++it;
    }
    return SG_OK;
}

static int retire(sg_server *s, int32_t *n_done)
{
    SgPool &p = s->pool;
    int32_t done = 0;
    for (auto it = s->rid_sid.begin(); it != s->rid_sid.end();) {
        const size_t slot = p.sid_slot.at(it->second);
        Request &r = *s->reqs[it->first];
        r.tick = p.scen[slot].tick;
        if (p.scen[slot].tick < p.scen[slot].horizon) {
            ++it;
            continue;
        }
        r.result.resize((size_t)r.d.n_agents);
        int rc = p.get_state(it->second, r.result.data(), r.d.n_agents);
        if (rc) return rc;
        p.release(it->second);
        s->resident_bytes -= r.bytes;
        r.status = SG_REQ_DONE;
        ++done;
        ++s->ndone;
        it = s->rid_sid.erase(it);
    }
    if (n_done) *n_done = done;
    return SG_OK;
}

extern "C" {

int sg_server_create(const sg_server_cfg *cfg, sg_server **out)
{
    if (!cfg || !out) return SG_ERR_INVALID;
    *out = nullptr;
    if (cfg->builtin != SG_BUILTIN_SIR_A && cfg->builtin != SG_BUILTIN_SIR_B) {
        sg_set_thread_error("sg_server_create: builtin must be SG_BUILTIN_SIR_A or SG_BUILTIN_SIR_B");
        return SG_ERR_INVALID;
    }
    if (cfg->budget_bytes <= 0 || cfg->agent_slots <= 0 || cfg->edge_slots < 0 || cfg->max_resident <= 0 ||
        cfg->agent_slots >= std::numeric_limits<int32_t>::max() ||
        cfg->edge_slots >= std::numeric_limits<int32_t>::max()) {
        sg_set_thread_error("sg_server_create: budget, slots or max_resident out of range");
        return SG_ERR_INVALID;
    }
    auto *s = new sg_server();
    s->cfg = *cfg;
    sg_engine_cfg ec{cfg->device, 0, cfg->stream};
    int rc = s->pool.init(&ec);
    // the pool keeps a logical-id array, so a request may carry its own RNG keys
    if (!rc) rc = s->pool.allocate(cfg->agent_slots, cfg->edge_slots, cfg->max_resident, false, true);
    if (rc) {
        sg_set_thread_error(s->pool.err);
        s->pool.destroy();
        delete s;
        return rc;
    }
    s->pool.builtin = cfg->builtin;
    *out = s;
    return SG_OK;
}

int sg_server_destroy(sg_server *s)
{
    if (!s) return SG_OK;
    s->pool.destroy();
    delete s;
    return SG_OK;
}

int sg_server_last_error(const sg_server *s, char *buf, size_t cap)
{
    if (!buf || !cap) return SG_ERR_INVALID;
    const std::string &m = s ? s->pool.err : std::string();
    const size_t k = std::min(cap - 1, m.size());
    memcpy(buf, m.data(), k);
    buf[k] = '\0';
    return SG_OK;
}

int sg_server_submit(sg_server *s, const sg_scenario_desc *d, int64_t *rid)
{
    if (!s || !d || !rid) return SG_ERR_INVALID;
    if (d->builtin != s->cfg.builtin) return s->pool.fail(SG_ERR_INVALID, "request builtin differs from the server's");
    if (!(d->flags & SG_GRAPH_SYMMETRIC)) return s->pool.fail(SG_ERR_INVALID, "the server takes symmetric (undirected) graphs");
    if (d->horizon < 0) return s->pool.fail(SG_ERR_INVALID, "horizon < 0");
    if (d->n_agents < 0 || d->nnz < 0 || !d->offsets || (d->nnz > 0 && !d->indices))
        return s->pool.fail(SG_ERR_INVALID, "bad CSR sizes or NULL arrays");
    if (!d->state && d->n_agents > 0) return s->pool.fail(SG_ERR_INVALID, "state is NULL");
    const int64_t bytes = sg_pool_scenario_bytes(d->n_agents, d->nnz, false, d->lids != nullptr);
    if (bytes > s->cfg.budget_bytes || d->n_agents + 1 > s->cfg.agent_slots || d->nnz > s->cfg.edge_slots)
        return s->pool.fail(SG_ERR_BUDGET, "request needs " + std::to_string((long long)bytes) +
                                               " bytes / slots beyond the server's budget or pool");
    if (d->offsets[0] != 0 || d->offsets[d->n_agents] != d->nnz)
        return s->pool.fail(SG_ERR_BAD_CSR, "offsets must start at 0 and end at nnz");
    // Nothing queued ahead and room now: placed on the device at once, straight
    // from the caller's arrays, with the CSR checked there (no host pass over
    // the edges). Otherwise the request is checked and copied on the host.
    if (s->queue.empty() && s->resident_bytes + bytes <= s->cfg.budget_bytes &&
        s->pool.fits(d->n_agents, d->nnz)) {
        const int32_t sid = s->next_sid++;
        const int rc = s->pool.place(*d, d->offsets, d->indices, d->state, d->lids, sid, true);
        if (rc == SG_OK) {
            auto r = std::make_unique<Request>();
            r->rid = s->next_rid++;
            r->d = *d;
            r->d.offsets = r->d.indices = r->d.state = nullptr;
            r->d.lids = nullptr;
            r->bytes = bytes;
            r->status = SG_REQ_RUNNING;
            *rid = r->rid;
            s->rid_sid[r->rid] = sid;
            s->resident_bytes += bytes;
            s->reqs[r->rid] = std::move(r);
            return SG_OK;
        }
        if (rc != SG_ERR_BUDGET) return rc; // SG_ERR_BAD_CSR from the device check, or a CUDA error
        // fragmented pool: queue it
    }
    if (d->flags & SG_REQ_BORROW) { // the caller keeps the arrays: no check or copy on the host
        auto r = std::make_unique<Request>();
        r->rid = s->next_rid++;
        r->d = *d;
        r->borrowed = true;
        r->bytes = bytes;
        *rid = r->rid;
        s->queue.push_back(r->rid);
        s->reqs[r->rid] = std::move(r);
        return SG_OK;
    }
    std::string why = sg_check_csr(d->offsets, d->n_agents, d->indices, d->nnz);
    if (!why.empty()) return s->pool.fail(SG_ERR_BAD_CSR, why);
    auto r = std::make_unique<Request>();
    r->rid = s->next_rid++;
    r->d = *d;
    r->off.assign(d->offsets, d->offsets + d->n_agents + 1);
    r->idx.assign(d->indices, d->indices + d->nnz);
    r->state.assign(d->state, d->state + d->n_agents);
    if (d->lids) r->lids.assign(d->lids, d->lids + d->n_agents);
    r->d.offsets = r->d.indices = r->d.state = nullptr;
    r->d.lids = nullptr;
    r->bytes = bytes;
    *rid = r->rid;
    s->queue.push_back(r->rid);
    s->reqs[r->rid] = std::move(r);
    return SG_OK;
}

int sg_server_step(sg_server *s, int32_t nticks, int32_t *n_done)
{
    if (!s || nticks < 0) return SG_ERR_INVALID;
    int rc = admit(s);
    if (rc) return rc;
    if (!s->rid_sid.empty()) {
        rc = s->pool.run(nticks, true);
        if (rc) return rc;
        cudaError_t ce = cudaStreamSynchronize(s->pool.stream);
        if (ce != cudaSuccess) return s->pool.cuda_fail(ce, "cudaStreamSynchronize");
    }
    return retire(s, n_done);
}

int sg_server_poll(sg_server *s, int64_t rid, int32_t *status, int64_t *tick)
{
    if (!s) return SG_ERR_INVALID;
    auto it = s->reqs.find(rid);
    if (it == s->reqs.end()) return s->pool.fail(SG_ERR_NOT_FOUND, "unknown request id");
    if (status) *status = it->second->status;
    if (tick) {
        auto rs = s->rid_sid.find(rid);
        *tick = rs == s->rid_sid.end() ? it->second->tick
                                       : s->pool.scen[s->pool.sid_slot.at(rs->second)].tick;
    }
    return SG_OK;
}

int sg_server_take_result(sg_server *s, int64_t rid, int32_t *host, int64_t n)
{
    if (!s || !host) return SG_ERR_INVALID;
    auto it = s->reqs.find(rid);
    if (it == s->reqs.end()) return s->pool.fail(SG_ERR_NOT_FOUND, "unknown request id");
    Request &r = *it->second;
    if (r.status == SG_REQ_FAILED) {
        const std::string why = r.failure;
        s->reqs.erase(it);
        return s->pool.fail(SG_ERR_BAD_CSR, "request refused when placed: " + why);
    }
    if (r.status != SG_REQ_DONE) return s->pool.fail(SG_ERR_INVALID, "request not finished");
    if (n != r.d.n_agents) return s->pool.fail(SG_ERR_INVALID, "n differs from the request's agent count");
    memcpy(host, r.result.data(), (size_t)n * 4);
    s->reqs.erase(it);
    return SG_OK;
}

int sg_server_counts(sg_server *s, int64_t *queued, int64_t *resident, int64_t *done, int64_t *resident_bytes)
{
    if (!s) return SG_ERR_INVALID;
    if (queued) *queued = (int64_t)s->queue.size();
    if (resident) *resident = (int64_t)s->rid_sid.size();
    if (done) *done = s->ndone;
    if (resident_bytes) *resident_bytes = s->resident_bytes;
    return SG_OK;
}

int sg_server_set_tune(sg_server *s, const sg_tune *t)
{
    if (!s || !t) return SG_ERR_INVALID;
    if (t->strategy != SG_SIR_PULL && t->strategy != SG_SIR_COUNT) return s->pool.fail(SG_ERR_INVALID, "bad strategy");
    if (t->blocks_per_sm < 1 || t->blocks_per_sm > 32 || t->thread_row < 1 || t->mega_row < 512 ||
        t->count_flavour < 0 || t->count_flavour > SG_FLAVOUR_MAX)
        return s->pool.fail(SG_ERR_INVALID, "tune parameters out of range");
    const bool mega_changed = t->mega_row != s->pool.tune.mega_row;
    s->pool.tune = *t;
    if (mega_changed) s->pool.tables_dirty = true;
    return SG_OK;
}

} // extern "C"
