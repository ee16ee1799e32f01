// sg_engine.cu -- the plain (single-scenario) engine behind the C ABI.
//
// Replaces SAGESim's per-simulate() path (sagesim/model.py:961-998 simulate,
// 1314-1640 worker_coroutine, 1020-1274 _build_gpu_buffers): the model is
// uploaded once into a structure-of-arrays property store (two buffers per
// double-buffered property), a device CSR and an RNG-key array; sg_run then
// issues one kernel per step per tick (plus the scatter of the count
// strategy) on one stream, with no host round trip between ticks. The
// reference's spin grid barriers (model.py:1956-1974) become stream order.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "sg_internal.h"
#include "sg_setup.h"
#include "sg_philox.h"
#include "sg_step_rt.h"

namespace {
thread_local std::string g_create_error;
// Rows longer than this are scanned by a whole block (see sg_kernels.cu).
constexpr int32_t kMegaRow = 2048;
}

struct SgProp {
    std::string name;
    int32_t dtype = SG_I32;
    int32_t width = 1;
    int64_t rows = 0; // agents, or the rows of a breed-local array
    bool dbuf = true;
    int cur = 0; // read buffer
    SgDev buf[2];
    SgDev snap;
    size_t row_bytes() const { return (size_t)width * 4; }
};

struct SgStep {
    int32_t id = 0;
    int32_t kind = 0; // SG_BUILTIN_* or 0 for a compiled step
    sg_builtin_params bp{};
    int32_t priority = 0;
    int64_t begin = 0, end = 0;
    std::vector<int32_t> written;
    SgCompiledStep *compiled = nullptr;
    // device tables
    SgDev seg, tiles, mega;
    int32_t ntiles = 0, nmega = 0;
    SgSeg host_seg{};
};

struct sg_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 152;
    size_t l2_window_max = 0; // largest access-policy window (bytes), 0 = unsupported
    size_t l2_limit_bytes = 0; // persisting-line capacity set for this context
    std::string err;

    int64_t n = -1, nnz = 0;
    int32_t graph_flags = 0;
    SgDev off, idx, toff, tidx;
    bool have_transpose = false;
    std::vector<int32_t> mega_agents; // agents whose row is longer than kMegaRow
    SgDev lids;
    bool has_lids = false;
    int64_t seed = 0;
    std::vector<double> globals;
    SgDev globals_dev;
    bool globals_dirty = true;

    std::vector<std::unique_ptr<SgProp>> props;
    std::vector<std::unique_ptr<SgStep>> steps;
    int32_t next_step_id = 0;

    // scratch of the count strategy and of per-tick statistics
    SgDev cnt, changes, change_rows, tile_nch, stats, chunks, nchunks, rowsegs, nrowsegs;
    SgDev cls, amask, mrebuild, tick_changes, tick_cand; // class sweep: classes, activity bits, per-tick counters
    bool cls_on = false;     // this run's count step keeps classes (its tiles start at multiples of 32)
    bool last_sweep = false; // the last run's count step was the class sweep
    SgDev flist[2], flen, fnch, fmark, fstats_init, fstats_delta; // frontier strategy
    SgDev transpose_tmp, scan_tmp;
    SgDev bm_radius, bm_rq, bm_trig; // opinion: Box-Muller tables, built once per engine
    bool bm_ready = false;
    SgDev nb8;               // opinion (width 8): first 8 neighbours per agent, group-major, -1 padded
    bool nb8_valid = false;  // nb8 matches the current graph
    bool l2_limit_set = false;
    SgDev prop_table; // sg_prop_dev per property, for compiled steps

    SgProfiler prof;
    int hub_deg = 32;
    sg_tune tune{SG_SIR_COUNT, 16, 32, 2048,
                 SG_FLAVOUR_SWEEP | SG_FLAVOUR_HYBRID | SG_FLAVOUR_FLAT | SG_FLAVOUR_DENSE | SG_FLAVOUR_LAZY, 0.0};
    int32_t last_nticks = 0;
    int64_t last_launches = 0; // kernels launched by the last enqueued run
    std::vector<int64_t> hist;  // per-tick S, I, R, E_S of consecutive runs with statistics
    int64_t hist_tick0 = 0;     // tick of hist's first row

    // CUDA graph of the tick loop (sg_run_async with use_graph)
    cudaGraphExec_t graph_exec = nullptr;
    int32_t graph_nticks = -1;
    uint64_t graph_version = 0;
    uint64_t version = 1; // bumped when steps/props/graph change

    int fail(int code, const std::string &msg)
    {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t ce, const char *what)
    {
        err = std::string(what) + ": " + cudaGetErrorString(ce);
        return ce == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
};

// Error message for calls without an engine handle (read with sg_last_error(NULL)).
void sg_set_thread_error(const std::string &msg) { g_create_error = msg; }

#define SG_CK(call)                                                                            \
    do {                                                                                       \
        cudaError_t _ce = (call);                                                              \
        if (_ce != cudaSuccess) return e->cuda_fail(_ce, #call);                               \
    } while (0)

std::string sg_check_csr(const int32_t *off, int64_t n, const int32_t *idx, int64_t nnz)
{
    char buf[256];
    if (n < 0 || n >= (int64_t)std::numeric_limits<int32_t>::max())
        return "agent count out of range";
    if (nnz < 0 || nnz >= (int64_t)std::numeric_limits<int32_t>::max())
        return "nnz out of range (int32 CSR)";
    if (!off) return "offsets is NULL";
    if (nnz > 0 && !idx) return "indices is NULL";
    if (off[0] != 0) return "offsets[0] != 0";
    for (int64_t i = 0; i < n; ++i) {
        if (off[i + 1] < off[i]) {
            snprintf(buf, sizeof buf, "offsets not monotone at row %lld", (long long)i);
            return buf;
        }
    }
    if ((int64_t)off[n] != nnz) {
        snprintf(buf, sizeof buf, "offsets[n] = %d but nnz = %lld", off[n], (long long)nnz);
        return buf;
    }
    for (int64_t k = 0; k < nnz; ++k) {
        if (idx[k] < 0 || (int64_t)idx[k] >= n) {
            snprintf(buf, sizeof buf, "index %d at entry %lld out of range [0, %lld)", idx[k],
                     (long long)k, (long long)n);
            return buf;
        }
    }
    return std::string();
}

extern "C" {

int sg_engine_create(const sg_engine_cfg *cfg, sg_engine **out)
{
    if (!out) {
        g_create_error = "out is NULL";
        return SG_ERR_INVALID;
    }
    *out = nullptr;
    int device = cfg ? cfg->device : 0;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev <= 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(ce);
        return SG_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) {
        g_create_error = "device ordinal out of range";
        return SG_ERR_INVALID;
    }
    ce = cudaSetDevice(device);
    if (ce != cudaSuccess) {
        g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(ce);
        return SG_ERR_CUDA;
    }
    auto *e = new sg_engine();
    e->device = device;
    e->sm_count = sg_sm_count(device);
    {
        int persist = 0, window = 0;
        if (cudaDeviceGetAttribute(&persist, cudaDevAttrMaxPersistingL2CacheSize, device) == cudaSuccess &&
            cudaDeviceGetAttribute(&window, cudaDevAttrMaxAccessPolicyWindowSize, device) == cudaSuccess &&
            persist > 0 && window > 0)
            e->l2_window_max = (size_t)std::min(persist, window);
        (void)cudaGetLastError();
    }
    if (cfg && cfg->stream) {
        e->stream = (cudaStream_t)cfg->stream;
    } else {
        ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
        if (ce != cudaSuccess) {
            g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(ce);
            delete e;
            return SG_ERR_CUDA;
        }
        e->own_stream = true;
    }
    *out = e;
    return SG_OK;
}

int sg_engine_destroy(sg_engine *e)
{
    if (!e) return SG_OK;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    e->prof.destroy();
    if (e->graph_exec) cudaGraphExecDestroy(e->graph_exec);
    for (auto &s : e->steps)
        if (s->compiled) sg_step_rt_destroy(s->compiled);
    e->steps.clear();
    e->props.clear();
    if (e->own_stream) cudaStreamDestroy(e->stream);
    delete e;
    return SG_OK;
}

int sg_last_error(const sg_engine *e, char *buf, size_t cap)
{
    if (!buf || cap == 0) return SG_ERR_INVALID;
    const std::string &m = e ? e->err : g_create_error;
    const size_t k = std::min(cap - 1, m.size());
    memcpy(buf, m.data(), k);
    buf[k] = '\0';
    return SG_OK;
}

int sg_set_graph_csr(sg_engine *e, const int32_t *offsets, int64_t n, const int32_t *indices,
                     int64_t nnz, int32_t flags)
{
    if (!e) return SG_ERR_INVALID;
    std::string why = sg_check_csr(offsets, n, indices, nnz);
    if (!why.empty()) return e->fail(SG_ERR_BAD_CSR, why);
    if (e->n >= 0 && e->n != n && !e->props.empty())
        return e->fail(SG_ERR_INVALID, "agent count differs from the existing properties");
    cudaSetDevice(e->device);
    SG_CK(e->off.reserve((size_t)(n + 1) * 4));
    SG_CK(e->idx.reserve((size_t)std::max<int64_t>(nnz, 1) * 4));
    SG_CK(cudaMemcpyAsync(e->off.p, offsets, (size_t)(n + 1) * 4, cudaMemcpyHostToDevice, e->stream));
    if (nnz > 0)
        SG_CK(cudaMemcpyAsync(e->idx.p, indices, (size_t)nnz * 4, cudaMemcpyHostToDevice, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    e->mega_agents.clear();
    for (int64_t i = 0; i < n; ++i)
        if (offsets[i + 1] - offsets[i] > kMegaRow) e->mega_agents.push_back((int32_t)i);
    for (auto &st : e->steps) st->ntiles = 0; // tile and mega tables are rebuilt
    e->n = n;
    e->nnz = nnz;
    e->graph_flags = flags;
    e->have_transpose = false;
    e->nb8_valid = false;
    e->version++;
    return SG_OK;
}

int sg_set_graph_id_edges(sg_engine *e, const int64_t *ids, int64_t n, const int64_t *src_ids,
                          const int64_t *dst_ids, int64_t nedges, int32_t flags)
{
    if (!e || (n > 0 && !ids) || (nedges > 0 && (!src_ids || !dst_ids))) return SG_ERR_INVALID;
    if (e->n >= 0 && e->n != n && !e->props.empty())
        return e->fail(SG_ERR_INVALID, "agent count differs from the existing properties");
    cudaSetDevice(e->device);
    int32_t *off = nullptr, *idx = nullptr;
    int64_t nnz = 0;
    std::string why;
    const int rc = sg_build_csr_from_ids(ids, n, src_ids, dst_ids, nedges, (flags & SG_GRAPH_SYMMETRIC) != 0,
                                         (flags & SG_GRAPH_ORDERED) != 0, e->stream, &off, &idx, &nnz, &why);
    if (rc != SG_OK) {
        if (off) cudaFree(off);
        if (idx) cudaFree(idx);
        return e->fail(rc, why);
    }
    if (nnz >= ((int64_t)1 << 31)) {
        cudaFree(off);
        cudaFree(idx);
        return e->fail(SG_ERR_INVALID, "more than 2^31 - 1 CSR entries");
    }
    e->off.release();
    e->idx.release();
    e->off.p = off;
    e->off.bytes = (size_t)(n + 1) * 4;
    e->idx.p = idx;
    e->idx.bytes = (size_t)std::max<int64_t>(nnz, 1) * 4;
    // long rows (mega agents) from the offsets
    std::vector<int32_t> hoff((size_t)n + 1);
    SG_CK(cudaMemcpy(hoff.data(), off, (size_t)(n + 1) * 4, cudaMemcpyDeviceToHost));
    e->mega_agents.clear();
    for (int64_t i = 0; i < n; ++i)
        if (hoff[(size_t)i + 1] - hoff[(size_t)i] > kMegaRow) e->mega_agents.push_back((int32_t)i);
    for (auto &st : e->steps) st->ntiles = 0; // tile and mega tables are rebuilt
    e->n = n;
    e->nnz = nnz;
    e->graph_flags = flags & (SG_GRAPH_SYMMETRIC | SG_GRAPH_ORDERED);
    e->have_transpose = false;
    e->nb8_valid = false;
    e->version++;
    return SG_OK;
}

int sg_get_graph_csr(sg_engine *e, int32_t *offsets, int32_t *indices, int64_t *nnz)
{
    if (!e || !nnz) return SG_ERR_INVALID;
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "no graph");
    cudaSetDevice(e->device);
    SG_CK(cudaStreamSynchronize(e->stream));
    if (offsets) SG_CK(cudaMemcpy(offsets, e->off.p, (size_t)(e->n + 1) * 4, cudaMemcpyDeviceToHost));
    if (indices && e->nnz > 0) SG_CK(cudaMemcpy(indices, e->idx.p, (size_t)e->nnz * 4, cudaMemcpyDeviceToHost));
    *nnz = e->nnz;
    return SG_OK;
}

int sg_set_logical_ids(sg_engine *e, const int64_t *lids, int64_t n)
{
    if (!e) return SG_ERR_INVALID;
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "set the graph before logical ids");
    if (n != e->n) return e->fail(SG_ERR_INVALID, "logical id count != agent count");
    cudaSetDevice(e->device);
    if (!lids) {
        e->has_lids = false;
        e->version++;
        return SG_OK;
    }
    // Philox keys on lid mod 2^32 (sagesim/math_utils.py:108), so 4 bytes per
    // agent carry the whole key.
    std::vector<uint32_t> k32((size_t)n);
    for (int64_t i = 0; i < n; ++i) k32[(size_t)i] = (uint32_t)(uint64_t)lids[i];
    SG_CK(e->lids.reserve((size_t)std::max<int64_t>(n, 1) * 4));
    SG_CK(cudaMemcpyAsync(e->lids.p, k32.data(), (size_t)n * 4, cudaMemcpyHostToDevice, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    e->has_lids = true;
    e->version++;
    return SG_OK;
}

int sg_set_seed(sg_engine *e, int64_t seed)
{
    if (!e) return SG_ERR_INVALID;
    e->seed = seed;
    e->version++;
    return SG_OK;
}

int sg_set_globals_f64(sg_engine *e, const double *values, int32_t n)
{
    if (!e || n < 0 || (n > 0 && !values)) return SG_ERR_INVALID;
    e->globals.assign(values, values + n);
    e->globals_dirty = true;
    return SG_OK;
}

static int add_prop(sg_engine *e, const char *name, int32_t dtype, int32_t width, int64_t rows,
                    int32_t double_buffered, const void *init, int32_t *prop_id)
{
    if (!e || !name || !prop_id) return SG_ERR_INVALID;
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "set the graph before adding properties");
    if (dtype != SG_I32 && dtype != SG_F32) return e->fail(SG_ERR_INVALID, "dtype must be SG_I32 or SG_F32");
    if (width < 1 || width > 4096) return e->fail(SG_ERR_INVALID, "width out of range");
    if (rows < 0 || rows > ((int64_t)1 << 31) - 1) return e->fail(SG_ERR_INVALID, "row count out of range");
    cudaSetDevice(e->device);
    auto p = std::make_unique<SgProp>();
    p->name = name;
    p->dtype = dtype;
    p->width = width;
    p->rows = rows;
    p->dbuf = double_buffered != 0;
    const size_t bytes = (size_t)std::max<int64_t>(rows, 1) * p->row_bytes();
    SG_CK(p->buf[0].reserve(bytes));
    if (p->dbuf) SG_CK(p->buf[1].reserve(bytes));
    if (init && rows > 0)
        SG_CK(cudaMemcpyAsync(p->buf[0].p, init, (size_t)rows * p->row_bytes(), cudaMemcpyHostToDevice,
                              e->stream));
    else
        SG_CK(cudaMemsetAsync(p->buf[0].p, 0, bytes, e->stream));
    if (p->dbuf) SG_CK(cudaMemsetAsync(p->buf[1].p, 0, bytes, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    *prop_id = (int32_t)e->props.size();
    e->props.push_back(std::move(p));
    e->version++;
    return SG_OK;
}

int sg_add_property(sg_engine *e, const char *name, int32_t dtype, int32_t width,
                    int32_t double_buffered, const void *init, int32_t *prop_id)
{
    if (!e) return SG_ERR_INVALID;
    return add_prop(e, name, dtype, width, e->n, double_buffered, init, prop_id);
}

int sg_add_array(sg_engine *e, const char *name, int32_t dtype, int32_t width, int64_t rows,
                 int32_t double_buffered, const void *init, int32_t *prop_id)
{
    if (!e) return SG_ERR_INVALID;
    return add_prop(e, name, dtype, width, rows, double_buffered, init, prop_id);
}

static int check_range(sg_engine *e, int32_t prop, int64_t first, int64_t count)
{
    if (prop < 0 || prop >= (int32_t)e->props.size()) return e->fail(SG_ERR_NOT_FOUND, "unknown property");
    if (first < 0 || count < 0 || first + count > e->props[prop]->rows)
        return e->fail(SG_ERR_INVALID, "row range out of bounds");
    return SG_OK;
}

int sg_set_property(sg_engine *e, int32_t prop, const void *host, int64_t first, int64_t count)
{
    if (!e) return SG_ERR_INVALID;
    int rc = check_range(e, prop, first, count);
    if (rc) return rc;
    if (count == 0) return SG_OK;
    if (!host) return e->fail(SG_ERR_INVALID, "host is NULL");
    cudaSetDevice(e->device);
    SgProp &p = *e->props[prop];
    char *dst = p.buf[p.cur].as<char>() + (size_t)first * p.row_bytes();
    SG_CK(cudaMemcpyAsync(dst, host, (size_t)count * p.row_bytes(), cudaMemcpyHostToDevice, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    return SG_OK;
}

int sg_get_property(sg_engine *e, int32_t prop, void *host, int64_t first, int64_t count)
{
    if (!e) return SG_ERR_INVALID;
    int rc = check_range(e, prop, first, count);
    if (rc) return rc;
    if (count == 0) return SG_OK;
    if (!host) return e->fail(SG_ERR_INVALID, "host is NULL");
    cudaSetDevice(e->device);
    SgProp &p = *e->props[prop];
    const char *src = p.buf[p.cur].as<char>() + (size_t)first * p.row_bytes();
    SG_CK(cudaMemcpyAsync(host, src, (size_t)count * p.row_bytes(), cudaMemcpyDeviceToHost, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    return SG_OK;
}

int sg_property_device_ptr(sg_engine *e, int32_t prop, void **dptr)
{
    if (!e || !dptr) return SG_ERR_INVALID;
    if (prop < 0 || prop >= (int32_t)e->props.size()) return e->fail(SG_ERR_NOT_FOUND, "unknown property");
    *dptr = e->props[prop]->buf[e->props[prop]->cur].p;
    return SG_OK;
}

int sg_add_builtin_step(sg_engine *e, const sg_builtin_params *bp, int32_t *step_id)
{
    if (!e || !bp) return SG_ERR_INVALID;
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "set the graph before adding steps");
    const int nprops = (int)e->props.size();
    if (bp->state_prop < 0 || bp->state_prop >= nprops)
        return e->fail(SG_ERR_NOT_FOUND, "state_prop is not a property");
    const SgProp &sp = *e->props[bp->state_prop];
    if (!sp.dbuf) return e->fail(SG_ERR_INVALID, "builtin steps need a double-buffered state property");
    if (sp.width != 1) return e->fail(SG_ERR_INVALID, "state property must have width 1");
    if (sp.rows != e->n) return e->fail(SG_ERR_INVALID, "state property must be an agent property, not an array");
    if (bp->begin < 0 || bp->end > e->n || bp->begin > bp->end)
        return e->fail(SG_ERR_INVALID, "step agent range out of bounds");
    if (bp->builtin == SG_BUILTIN_SIR_A || bp->builtin == SG_BUILTIN_SIR_B) {
        if (sp.dtype != SG_I32) return e->fail(SG_ERR_INVALID, "SIR state must be int32");
        if (bp->strategy != SG_SIR_PULL && bp->strategy != SG_SIR_COUNT && bp->strategy != SG_SIR_FRONTIER)
            return e->fail(SG_ERR_INVALID, "unknown SIR strategy");
    } else if (bp->builtin == SG_BUILTIN_OPINION) {
        if (sp.dtype != SG_F32) return e->fail(SG_ERR_INVALID, "opinion must be float32");
        if (bp->aux_prop < 0 || bp->aux_prop >= nprops || e->props[bp->aux_prop]->dtype != SG_F32 ||
            e->props[bp->aux_prop]->rows != e->n)
            return e->fail(SG_ERR_INVALID, "opinion needs a float32 weights property (aux_prop)");
    } else {
        return e->fail(SG_ERR_INVALID, "unknown builtin");
    }
    for (auto &s : e->steps)
        if (s->kind == SG_BUILTIN_SIR_A || s->kind == SG_BUILTIN_SIR_B)
            if ((bp->builtin == SG_BUILTIN_SIR_A || bp->builtin == SG_BUILTIN_SIR_B) &&
                s->bp.strategy != SG_SIR_PULL && bp->strategy != SG_SIR_PULL)
                return e->fail(SG_ERR_INVALID, "one count- or frontier-strategy SIR step per engine");
    auto s = std::make_unique<SgStep>();
    s->id = e->next_step_id++;
    s->kind = bp->builtin;
    s->bp = *bp;
    s->priority = bp->priority;
    s->begin = bp->begin;
    s->end = bp->end;
    s->written.push_back(bp->state_prop);
    *step_id = s->id;
    e->steps.push_back(std::move(s));
    e->version++;
    return SG_OK;
}

int sg_update_builtin_step(sg_engine *e, int32_t step_id, const sg_builtin_params *bp)
{
    if (!e || !bp) return SG_ERR_INVALID;
    for (auto &s : e->steps) {
        if (s->id != step_id) continue;
        if (s->kind == 0 || s->kind != bp->builtin || s->bp.state_prop != bp->state_prop ||
            s->bp.aux_prop != bp->aux_prop || s->bp.strategy != bp->strategy ||
            s->begin != bp->begin || s->end != bp->end)
            return e->fail(SG_ERR_INVALID, "update may change only probabilities, codes and priority");
        s->bp = *bp;
        s->priority = bp->priority;
        e->version++;
        return SG_OK;
    }
    return e->fail(SG_ERR_NOT_FOUND, "unknown step id");
}

int sg_compile_step(sg_engine *e, const char *cuda_src, const char *entry, int32_t priority,
                    int64_t begin, int64_t end, const int32_t *written_props, int32_t n_written,
                    int32_t *step_id)
{
    if (!e || !cuda_src || !entry || !step_id || n_written < 0) return SG_ERR_INVALID;
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "set the graph before adding steps");
    if (begin < 0 || end > e->n || begin > end) return e->fail(SG_ERR_INVALID, "step agent range out of bounds");
    for (int i = 0; i < n_written; ++i)
        if (written_props[i] < 0 || written_props[i] >= (int32_t)e->props.size())
            return e->fail(SG_ERR_NOT_FOUND, "written property id out of range");
    std::string log;
    cudaSetDevice(e->device);
    SgCompiledStep *cs = nullptr;
    int rc = sg_step_rt_compile(e->device, cuda_src, entry, &cs, &log);
    if (rc != SG_OK) return e->fail(rc, log);
    auto s = std::make_unique<SgStep>();
    s->id = e->next_step_id++;
    s->kind = 0;
    s->priority = priority;
    s->begin = begin;
    s->end = end;
    s->written.assign(written_props, written_props + n_written);
    s->compiled = cs;
    *step_id = s->id;
    e->steps.push_back(std::move(s));
    e->version++;
    return SG_OK;
}

// ---- execution ------------------------------------------------------------------

struct SgPlan {
    std::vector<SgStep *> order;             // by (priority, insertion)
    std::vector<int32_t> copy_props;         // double-buffered props needing copy-through
    std::vector<int32_t> swap_props;         // double-buffered props written this tick
    SgStep *count_step = nullptr; // the SIR step keeping infected-neighbour counts
    bool count_inplace = false;   // it is the only step: state updated in place
    bool frontier = false;        // it uses the frontier strategy
};

static SgPlan make_plan(sg_engine *e)
{
    SgPlan pl;
    for (auto &s : e->steps) pl.order.push_back(s.get());
    std::stable_sort(pl.order.begin(), pl.order.end(),
                     [](const SgStep *a, const SgStep *b) { return a->priority < b->priority; });
    std::vector<int> written(e->props.size(), 0);
    std::vector<int> fully(e->props.size(), 0);
    for (SgStep *s : pl.order) {
        for (int32_t p : s->written) {
            if (!e->props[p]->dbuf) continue;
            written[p]++;
            // a builtin writes every agent of its range; one covering all agents
            // and the only writer needs no copy-through
            if (s->kind != 0 && s->begin == 0 && s->end == e->n) fully[p]++;
        }
        if ((s->kind == SG_BUILTIN_SIR_A || s->kind == SG_BUILTIN_SIR_B) &&
            s->bp.strategy != SG_SIR_PULL)
            pl.count_step = s;
    }
    pl.count_inplace = pl.count_step != nullptr && pl.order.size() == 1;
    pl.frontier = pl.count_step != nullptr && pl.count_step->bp.strategy == SG_SIR_FRONTIER;
    for (size_t p = 0; p < e->props.size(); ++p) {
        if (!written[p]) continue;
        if (pl.count_inplace && (int32_t)p == pl.count_step->bp.state_prop) continue;
        pl.swap_props.push_back((int32_t)p);
        if (!(written[p] == 1 && fully[p] == 1)) pl.copy_props.push_back((int32_t)p);
    }
    return pl;
}

// Fills the step's segment for a run starting at tick0 and uploads it.
static int prepare_step(sg_engine *e, SgStep *s, int64_t tick0, unsigned long long *stats)
{
    SgSeg &g = s->host_seg;
    memset(&g, 0, sizeof g);
    g.tick0 = tick0;
    g.end_tick = std::numeric_limits<int64_t>::max();
    g.lids = e->has_lids ? e->lids.as<uint32_t>() : nullptr;
    g.lid_base = 0;
    g.key = (uint32_t)(uint64_t)e->seed;
    if (s->kind != 0) {
        const SgProp &sp = *e->props[s->bp.state_prop];
        g.par0 = sp.cur;
        g.variant = s->kind;
        g.kinf = sg_threshold_host(s->bp.beta);
        g.krec = sg_threshold_host(s->bp.gamma);
        g.cs = s->bp.code_s;
        g.ci = s->bp.code_i;
        g.cr = s->bp.code_r;
        g.stats = (s->kind == SG_BUILTIN_OPINION) ? nullptr : stats;
        if (s->kind == SG_BUILTIN_OPINION) {
            const SgProp &wp = *e->props[s->bp.aux_prop];
            g.width = wp.width;
            g.sigma = s->bp.sigma;
            g.weights = wp.buf[wp.cur].as<float>();
        }
    }
    if (!s->tiles.p || s->ntiles == 0) {
        std::vector<SgTile> tiles;
        sg_append_tiles(tiles, 0, s->begin, s->end);
        s->ntiles = (int32_t)tiles.size();
        SG_CK(s->tiles.reserve(std::max<size_t>(tiles.size(), 1) * sizeof(SgTile)));
        if (!tiles.empty())
            SG_CK(cudaMemcpyAsync(s->tiles.p, tiles.data(), tiles.size() * sizeof(SgTile),
                                  cudaMemcpyHostToDevice, e->stream));
        std::vector<SgMega> mg;
        for (int32_t a : e->mega_agents)
            if (a >= s->begin && a < s->end) mg.push_back(SgMega{a, 0});
        s->nmega = (int32_t)mg.size();
        SG_CK(s->mega.reserve(std::max<size_t>(mg.size(), 1) * sizeof(SgMega)));
        if (!mg.empty())
            SG_CK(cudaMemcpyAsync(s->mega.p, mg.data(), mg.size() * sizeof(SgMega),
                                  cudaMemcpyHostToDevice, e->stream));
    }
    SG_CK(s->seg.reserve(sizeof(SgSeg)));
    SG_CK(cudaMemcpyAsync(s->seg.p, &g, sizeof g, cudaMemcpyHostToDevice, e->stream));
    return SG_OK;
}

static int ensure_transpose(sg_engine *e)
{
    if (e->have_transpose || (e->graph_flags & SG_GRAPH_SYMMETRIC)) return SG_OK;
    SG_CK(e->toff.reserve((size_t)(e->n + 1) * 4));
    SG_CK(e->tidx.reserve((size_t)std::max<int64_t>(e->nnz, 1) * 4));
    SG_CK(e->transpose_tmp.reserve((size_t)(e->n + 1) * 4));
    const size_t sb = sg_transpose_scan_bytes(e->n);
    SG_CK(e->scan_tmp.reserve(std::max<size_t>(sb, 16)));
    SG_CK(sg_transpose_csr(e->off.as<int32_t>(), e->idx.as<int32_t>(), e->n, e->nnz,
                           e->toff.as<int32_t>(), e->tidx.as<int32_t>(),
                           e->transpose_tmp.as<int32_t>(), e->scan_tmp.p, e->scan_tmp.bytes,
                           e->stream));
    e->have_transpose = true;
    return SG_OK;
}

static SgTickArgs base_args(sg_engine *e, SgStep *s, int32_t r, bool inplace)
{
    SgTickArgs a{};
    a.off = e->off.as<int32_t>();
    a.idx = e->idx.as<int32_t>();
    if (s->kind != 0) {
        SgProp &sp = *e->props[s->bp.state_prop];
        a.buf0 = inplace ? sp.buf[sp.cur].p : sp.buf[0].p;
        a.buf1 = inplace ? sp.buf[sp.cur].p : sp.buf[1].p;
    }
    a.segs = s->seg.as<SgSeg>();
    a.tiles = s->tiles.as<SgTile>();
    a.ntiles = s->ntiles;
    a.r = r;
    a.thread_row = e->tune.thread_row;
    a.flavour = e->tune.count_flavour;
    a.sweep_wpt = sg_sweep_wpt(s->ntiles, e->sm_count, a.flavour);
    sg_hybrid_thresholds(s->ntiles, e->sm_count, a.flavour, &a.hybrid_rise, &a.hybrid_fall);
    if ((a.flavour & SG_FLAVOUR_SWEEP) && !(a.flavour & SG_FLAVOUR_FORCE) &&
        s->ntiles < e->sm_count * SG_SWEEP_MIN_TILES_PER_SM)
        a.flavour = (a.flavour & ~SG_FLAVOUR_SWEEP) | SG_FLAVOUR_LAZY;
    a.mega = s->mega.as<SgMega>();
    a.nmega = s->nmega;
    a.mega_blocks = std::min(s->nmega, e->sm_count);
    a.mega_row = kMegaRow;
    a.cnt = e->cnt.as<int32_t>();
    if (e->cls_on && s->bp.strategy == SG_SIR_COUNT)
        a.cnt_window = std::min(e->l2_window_max, (size_t)e->n * sizeof(int32_t));
    a.changes = e->changes.as<int32_t>();
    a.change_rows = s->bp.strategy == SG_SIR_COUNT ? e->change_rows.as<int2>() : nullptr;
    a.tile_nch = e->tile_nch.as<int32_t>();
    a.chunks = e->chunks.as<SgChunk>();
    a.nchunks = e->nchunks.as<int32_t>();
    a.rowsegs = e->rowsegs.as<SgRowSeg>();
    a.nrowsegs = e->nrowsegs.as<int32_t>();
    if (e->cls_on && s->bp.strategy == SG_SIR_COUNT &&
        (s->kind == SG_BUILTIN_SIR_A || s->kind == SG_BUILTIN_SIR_B)) {
        a.cls = e->cls.as<uint8_t>();
        a.amask = e->amask.as<uint32_t>();
        a.mrebuild = e->mrebuild.as<uint8_t>();
        a.tick_changes = e->tick_changes.as<int32_t>();
        a.tick_cand = e->tick_cand.as<int32_t>();
    }
    const bool sym = (e->graph_flags & SG_GRAPH_SYMMETRIC) != 0;
    a.toff = sym ? e->off.as<int32_t>() : e->toff.as<int32_t>();
    a.tidx = sym ? e->idx.as<int32_t>() : e->tidx.as<int32_t>();
    a.list[0] = e->flist[0].as<int32_t>();
    a.list[1] = e->flist[1].as<int32_t>();
    a.list_len = e->flen.as<int32_t>();
    a.nch = e->fnch.as<int32_t>();
    a.mark = e->fmark.as<int32_t>();
    a.aseg = nullptr;
    a.stats_init = e->fstats_init.as<unsigned long long>();
    a.stats_delta = e->fstats_delta.as<unsigned long long>();
    return a;
}

static int grid_for(sg_engine *e, int32_t ntiles)
{
    const int cap = e->sm_count * std::max(e->tune.blocks_per_sm, 1);
    return std::max(1, std::min(ntiles, cap));
}

#define SG_PROF_LAUNCH(kindname, launch_expr)                                                  \
    do {                                                                                       \
        size_t _tok = 0;                                                                       \
        const bool _p = e->prof.on && !capturing;                                              \
        if (_p) _tok = e->prof.begin(e->prof.kind(kindname), e->stream);                      \
        cudaError_t _ce = (launch_expr);                                                       \
        if (_ce != cudaSuccess) return e->cuda_fail(_ce, kindname);                            \
        if (_p) e->prof.end(_tok, e->stream);                                                  \
        ++e->last_launches;                                                                    \
    } while (0)

// Infected-neighbour counts at the run start. A step over every agent counts by
// scattering from the infected agents (two kernels; work = their degree sum),
// any other by scanning its agents' rows.
static cudaError_t launch_count_init(sg_engine *e, const SgStep *s, const SgTickArgs &a)
{
    if (s->begin == 0 && s->end == e->n) {
        ++e->last_launches; // two kernels
        return sg_launch_sir_count_init_scatter(a, grid_for(e, s->ntiles), e->stream);
    }
    return sg_launch_sir_count_init(a, grid_for(e, s->ntiles) + a.mega_blocks, e->stream);
}

// Enqueues nticks ticks (relative ticks 0..nticks-1) for the prepared steps.
static int enqueue_ticks(sg_engine *e, const SgPlan &pl, int32_t nticks, bool stats_on,
                         bool capturing)
{
    e->last_launches = 0;
    const int grid_sc = e->sm_count * 16;
    if (pl.frontier) {
        SgStep *s = pl.count_step;
        SgTickArgs a = base_args(e, s, 0, true);
        const int variant = s->kind == SG_BUILTIN_SIR_A ? 1 : 2;
        const int fgrid = e->sm_count * 8;
        SG_CK(cudaMemsetAsync(e->flen.p, 0, (size_t)(nticks + 1) * 4, e->stream));
        SG_CK(cudaMemsetAsync(e->fnch.p, 0, (size_t)std::max(nticks, 1) * 4, e->stream));
        if (stats_on) {
            SG_CK(cudaMemsetAsync(e->fstats_init.p, 0, 4 * 8, e->stream));
            SG_CK(cudaMemsetAsync(e->fstats_delta.p, 0, (size_t)std::max(nticks, 1) * 32, e->stream));
        }
        SG_PROF_LAUNCH("sir_count_init", launch_count_init(e, s, a));
        SG_PROF_LAUNCH("frontier_build", sg_launch_frontier_build(a, stats_on, grid_for(e, s->ntiles), e->stream));
        for (int32_t r = 0; r < nticks; ++r) {
            a.r = r;
            SG_PROF_LAUNCH("frontier_step", sg_launch_frontier_step(a, variant, stats_on, fgrid, e->stream));
            SG_PROF_LAUNCH("frontier_scatter", sg_launch_frontier_scatter(a, fgrid, e->stream));
        }
        return SG_OK;
    }
    if (pl.count_step) {
        SgStep *s = pl.count_step;
        SgTickArgs a = base_args(e, s, 0, pl.count_inplace);
        SG_CK(cudaMemsetAsync(e->nchunks.p, 0, (size_t)std::max(nticks, 1) * 4, e->stream));
        SG_CK(cudaMemsetAsync(e->nrowsegs.p, 0, (size_t)std::max(nticks, 1) * 4, e->stream));
        if (e->cls_on) { // the init builds exact activity bits: no rebuild at r == 0
            SG_CK(cudaMemsetAsync(e->mrebuild.p, 0, (size_t)nticks + 1, e->stream));
            SG_CK(cudaMemsetAsync(e->tick_changes.p, 0, (size_t)std::max(nticks, 1) * 4, e->stream));
            SG_CK(cudaMemsetAsync(e->tick_cand.p, 0, (size_t)std::max(nticks, 1) * 4, e->stream));
        }
        SG_PROF_LAUNCH("sir_count_init", launch_count_init(e, s, a));
    }
    for (int32_t r = 0; r < nticks; ++r) {
        for (int32_t p : pl.copy_props) {
            SgProp &pp = *e->props[p];
            const int rd = (pp.cur + r) & 1;
            SG_PROF_LAUNCH("copy_through",
                           sg_launch_copy_words(pp.buf[rd].as<uint32_t>(), pp.buf[rd ^ 1].as<uint32_t>(),
                                                pp.rows * pp.width, e->stream));
        }
        for (SgStep *s : pl.order) {
            const bool inplace = pl.count_inplace && s == pl.count_step;
            SgTickArgs a = base_args(e, s, r, inplace);
            const int grid = grid_for(e, s->ntiles);
            if (s->kind == SG_BUILTIN_SIR_A || s->kind == SG_BUILTIN_SIR_B) {
                const int variant = s->kind == SG_BUILTIN_SIR_A ? 1 : 2;
                if (s->bp.strategy == SG_SIR_COUNT) {
                    int nk = 1;
                    SG_PROF_LAUNCH("sir_count_step",
                                   sg_launch_sir_count_step(a, variant, stats_on, inplace, grid, e->stream, &nk));
                    e->last_launches += nk - 1;
                    SG_PROF_LAUNCH("sir_count_scatter", sg_launch_sir_count_scatter(a, grid_sc, e->stream));
                } else {
                    SG_PROF_LAUNCH("sir_pull",
                                   sg_launch_sir_pull(a, variant, stats_on, grid + a.mega_blocks, e->stream));
                }
            } else if (s->kind == SG_BUILTIN_OPINION) {
                a.bm_radius = e->bm_ready ? e->bm_radius.as<float2>() : nullptr;
                a.bm_rq = e->bm_ready ? e->bm_rq.as<uint32_t>() : nullptr;
                a.bm_trig = e->bm_ready ? e->bm_trig.as<float2>() : nullptr;
                a.nb8 = e->nb8_valid && s->host_seg.width == 8 ? e->nb8.as<int32_t>() : nullptr;
                {
                    const double sg = s->bp.sigma;
                    a.sigma_hi = (float)sg;
                    a.sigma_lo = (float)(sg - (double)a.sigma_hi);
                }
                if (e->bm_ready && e->l2_limit_bytes) {
                    a.l2_win = a.bm_rq;
                    a.l2_win_bytes = std::min(e->l2_window_max, SG_BM_RQ_BYTES);
                    a.l2_win_hit = (float)std::min(1.0, (double)e->l2_limit_bytes / (double)a.l2_win_bytes);
                }
                SG_PROF_LAUNCH("opinion", sg_launch_opinion(a, grid, e->stream, s->host_seg.width));
            } else {
                sg_step_args L{};
                L.tiles = (const int *)s->tiles.p;
                L.ntiles = s->ntiles;
                L.r = r;
                L.tick0 = s->host_seg.tick0;
                L.key = s->host_seg.key;
                L.nprops = (int)e->props.size();
                L.lids = (const unsigned int *)(e->has_lids ? e->lids.p : nullptr);
                L.off = e->off.as<int32_t>();
                L.idx = e->idx.as<int32_t>();
                L.g = e->globals_dev.as<double>();
                L.props = e->prop_table.as<sg_prop_dev>();
                L.n = e->n;
                SG_PROF_LAUNCH("compiled_step", sg_step_rt_launch(s->compiled, L, grid, e->stream));
            }
        }
    }
    return SG_OK;
}

static int upload_globals(sg_engine *e)
{
    if (!e->globals_dirty) return SG_OK;
    const size_t bytes = std::max<size_t>(e->globals.size(), 1) * sizeof(double);
    SG_CK(e->globals_dev.reserve(bytes));
    if (!e->globals.empty())
        SG_CK(cudaMemcpyAsync(e->globals_dev.p, e->globals.data(), e->globals.size() * sizeof(double),
                              cudaMemcpyHostToDevice, e->stream));
    e->globals_dirty = false;
    return SG_OK;
}

static int prepare_run(sg_engine *e, const SgPlan &pl, int64_t tick0, int32_t nticks, bool stats_on)
{
    int rc = upload_globals(e);
    if (rc) return rc;
    unsigned long long *stats = nullptr;
    if (stats_on) {
        SG_CK(e->stats.reserve((size_t)std::max(nticks, 1) * 4 * sizeof(unsigned long long)));
        SG_CK(cudaMemsetAsync(e->stats.p, 0, (size_t)std::max(nticks, 1) * 4 * 8, e->stream));
        stats = e->stats.as<unsigned long long>();
    }
    if (pl.count_step) {
        rc = ensure_transpose(e);
        if (rc) return rc;
        SG_CK(e->cnt.reserve((size_t)std::max<int64_t>(e->n, 1) * 4));
        SG_CK(e->changes.reserve((size_t)std::max<int64_t>(e->n, 1) * 4));
        SG_CK(e->change_rows.reserve((size_t)std::max<int64_t>(e->n, 1) * sizeof(int2)));
    }
    if (pl.frontier) {
        if (!pl.count_inplace)
            return e->fail(SG_ERR_INVALID, "the frontier strategy needs the SIR step to be the engine's only step");
        const size_t nb = (size_t)std::max<int64_t>(e->n, 1) * 4;
        SG_CK(e->flist[0].reserve(nb));
        SG_CK(e->flist[1].reserve(nb));
        SG_CK(e->fmark.reserve(nb));
        SG_CK(e->flen.reserve((size_t)(nticks + 1) * 4));
        SG_CK(e->fnch.reserve((size_t)std::max(nticks, 1) * 4));
        SG_CK(e->fstats_init.reserve(4 * 8));
        SG_CK(e->fstats_delta.reserve((size_t)std::max(nticks, 1) * 32));
    }
    {
        // property views of compiled steps; cur0 fixes the parity at r == 0. A
        // double-buffered property that no step of the run writes keeps its
        // current buffer for the whole run (its other buffer is not kept up to date).
        std::vector<sg_prop_dev> tab;
        for (size_t k = 0; k < e->props.size(); ++k) {
            const SgProp &p = *e->props[k];
            const bool swaps = p.dbuf && std::find(pl.swap_props.begin(), pl.swap_props.end(), (int32_t)k) !=
                                             pl.swap_props.end();
            if (swaps)
                tab.push_back(sg_prop_dev{p.buf[0].p, p.buf[1].p, p.width, 1, p.cur, p.dtype, (long long)p.rows});
            else
                tab.push_back(sg_prop_dev{p.buf[p.cur].p, p.buf[p.cur].p, p.width, 0, 0, p.dtype, (long long)p.rows});
        }
        SG_CK(e->prop_table.reserve(std::max<size_t>(tab.size(), 1) * sizeof(sg_prop_dev)));
        if (!tab.empty())
            SG_CK(cudaMemcpyAsync(e->prop_table.p, tab.data(), tab.size() * sizeof(sg_prop_dev),
                                  cudaMemcpyHostToDevice, e->stream));
    }
    for (SgStep *s : pl.order) {
        rc = prepare_step(e, s, tick0, stats);
        if (rc) return rc;
        if (s->kind == SG_BUILTIN_OPINION && !e->bm_ready) { // before any capture
            SG_CK(e->bm_radius.reserve((size_t)SG_BOX_MULLER_SIZE * sizeof(float2)));
            SG_CK(e->bm_rq.reserve(SG_BM_RQ_BYTES));
            SG_CK(e->bm_trig.reserve((size_t)SG_BM_TRIG_ENTRIES * sizeof(float2)));
            SG_CK(sg_launch_opinion_tables(e->bm_radius.as<float2>(), e->bm_rq.as<uint32_t>(),
                                           e->bm_trig.as<float2>(), e->stream));
            e->bm_ready = true;
        }
        if (s->kind == SG_BUILTIN_OPINION && s->host_seg.width == 8 && !e->nb8_valid && e->n > 0) {
            // the neighbour table of the width-8 opinion step, rebuilt with the graph
            SG_CK(e->nb8.reserve((size_t)SG_NB8_ENTRIES(e->n) * sizeof(int32_t)));
            SG_CK(sg_launch_opinion_neighbours8(e->off.as<int32_t>(), e->idx.as<int32_t>(), e->n,
                                                e->nb8.as<int32_t>(), e->stream));
            e->nb8_valid = true;
        }
    }
    if (pl.count_step) {
        SG_CK(e->tile_nch.reserve((size_t)std::max(pl.count_step->ntiles, 1) * 4));
        SG_CK(e->chunks.reserve(((size_t)e->n / 32 + pl.count_step->ntiles + 1) * sizeof(SgChunk)));
        SG_CK(e->nchunks.reserve((size_t)std::max(nticks, 1) * 4));
        SG_CK(e->rowsegs.reserve(SG_ROWSEG_CAPACITY(e->nnz) * sizeof(SgRowSeg)));
        SG_CK(e->nrowsegs.reserve((size_t)std::max(nticks, 1) * 4));
    }
    // class bytes and activity bits: kept by every count-strategy kernel, read by
    // the class sweep; a mask word belongs to one tile only if tiles start at
    // multiples of 32
    e->cls_on = pl.count_step && !pl.frontier && pl.count_step->begin % 32 == 0;
    if (e->cls_on) {
        SG_CK(e->cls.reserve(((size_t)e->n + 16) & ~size_t(15)));
        SG_CK(e->amask.reserve(((size_t)e->n / 32 + 2) * 4));
        SG_CK(e->mrebuild.reserve((size_t)nticks + 1));
        SG_CK(e->tick_changes.reserve((size_t)std::max(nticks, 1) * 4));
        SG_CK(e->tick_cand.reserve((size_t)std::max(nticks, 1) * 4));
    }
    if (e->cls_on && e->l2_window_max && !e->l2_limit_set) {
        // persisting-line capacity of this context (ends with it) for the counts' window
        e->l2_limit_bytes = std::min(e->l2_window_max, (size_t)e->n * 4);
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, e->l2_limit_bytes);
        (void)cudaGetLastError();
        e->l2_limit_set = true;
    }
    if (e->bm_ready && e->l2_window_max && !e->l2_limit_set) {
        // the opinion step's radius corrections (32 MiB, read at random) as persisting lines
        e->l2_limit_bytes = std::min(e->l2_window_max, SG_BM_RQ_BYTES);
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, e->l2_limit_bytes);
        (void)cudaGetLastError();
        e->l2_limit_set = true;
    }
    e->last_sweep = e->cls_on && pl.count_inplace && (e->tune.count_flavour & SG_FLAVOUR_SWEEP) &&
                    ((e->tune.count_flavour & SG_FLAVOUR_FORCE) ||
                     pl.count_step->ntiles >= e->sm_count * SG_SWEEP_MIN_TILES_PER_SM);
    return SG_OK;
}

static void finish_run(sg_engine *e, const SgPlan &pl, int32_t nticks)
{
    e->last_nticks = nticks;
    for (int32_t p : pl.swap_props) e->props[p]->cur = (e->props[p]->cur + nticks) & 1;
}

int sg_run(sg_engine *e, int64_t tick0, int32_t nticks, int64_t *tick_stats, sg_stats *out)
{
    if (!e) return SG_ERR_INVALID;
    if (nticks < 0) return e->fail(SG_ERR_INVALID, "nticks < 0");
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "no graph");
    cudaSetDevice(e->device);
    SgPlan pl = make_plan(e);
    const bool stats_on = tick_stats != nullptr || out != nullptr;
    int rc = prepare_run(e, pl, tick0, nticks, stats_on);
    if (rc) return rc;
    cudaEvent_t t0, t1;
    SG_CK(cudaEventCreate(&t0));
    SG_CK(cudaEventCreate(&t1));
    SG_CK(cudaEventRecord(t0, e->stream));
    rc = enqueue_ticks(e, pl, nticks, stats_on, false);
    if (rc) {
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        return rc;
    }
    SG_CK(cudaEventRecord(t1, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (e->prof.on) e->prof.collect();
    finish_run(e, pl, nticks);

    std::vector<unsigned long long> st;
    if (stats_on && nticks > 0) {
        st.resize((size_t)nticks * 4);
        if (pl.frontier) {
            // deltas per tick -> absolute S, I, R after the tick and E_S at its start
            unsigned long long init[4];
            std::vector<unsigned long long> d((size_t)nticks * 4);
            SG_CK(cudaMemcpy(init, e->fstats_init.p, sizeof init, cudaMemcpyDeviceToHost));
            SG_CK(cudaMemcpy(d.data(), e->fstats_delta.p, d.size() * 8, cudaMemcpyDeviceToHost));
            unsigned long long S = init[0], I = init[1], R = init[2], ES = init[3];
            for (int32_t r = 0; r < nticks; ++r) {
                const unsigned long long inf = d[(size_t)r * 4], rec = d[(size_t)r * 4 + 1],
                                         deg = d[(size_t)r * 4 + 2];
                st[(size_t)r * 4 + 3] = ES;
                S -= inf;
                I = I + inf - rec;
                R += rec;
                ES -= deg;
                st[(size_t)r * 4] = S;
                st[(size_t)r * 4 + 1] = I;
                st[(size_t)r * 4 + 2] = R;
            }
        } else {
            SG_CK(cudaMemcpy(st.data(), e->stats.p, st.size() * 8, cudaMemcpyDeviceToHost));
        }
        if (tick_stats)
            for (size_t k = 0; k < st.size(); ++k) tick_stats[k] = (int64_t)st[k];
        // a run that does not continue the recorded ticks starts a new history
        if (tick0 != e->hist_tick0 + (int64_t)(e->hist.size() / 4)) {
            e->hist.clear();
            e->hist_tick0 = tick0;
        }
        for (unsigned long long v : st) e->hist.push_back((int64_t)v);
    }
    if (out) {
        out->ticks = nticks;
        int64_t agents = 0;
        for (SgStep *s : pl.order)
            if (s->kind == SG_BUILTIN_SIR_A || s->kind == SG_BUILTIN_SIR_B) agents += s->end - s->begin;
        out->agent_ticks = agents * nticks;
        int64_t ev = 0;
        for (int32_t r = 0; r < nticks; ++r) ev += (int64_t)st[(size_t)r * 4 + 3];
        out->edge_visits = ev;
        out->device_ms = ms;
        out->kernel_launches = e->last_launches;
    }
    return SG_OK;
}

int sg_get_tick_history(sg_engine *e, int64_t *out, int64_t max_ticks, int64_t *nticks, int64_t *first_tick)
{
    if (!e || max_ticks < 0) return SG_ERR_INVALID;
    const int64_t rows = (int64_t)(e->hist.size() / 4);
    if (nticks) *nticks = rows;
    if (first_tick) *first_tick = e->hist_tick0;
    const int64_t k = std::min(rows, max_ticks);
    if (out && k > 0) memcpy(out, e->hist.data(), (size_t)k * 4 * sizeof(int64_t));
    return SG_OK;
}

int sg_run_async(sg_engine *e, int64_t tick0, int32_t nticks, int32_t use_graph)
{
    if (!e) return SG_ERR_INVALID;
    if (nticks < 0) return e->fail(SG_ERR_INVALID, "nticks < 0");
    if (e->n < 0) return e->fail(SG_ERR_INVALID, "no graph");
    cudaSetDevice(e->device);
    SgPlan pl = make_plan(e);
    int rc = prepare_run(e, pl, tick0, nticks, false);
    if (rc) return rc;
    if (!use_graph) {
        rc = enqueue_ticks(e, pl, nticks, false, false);
        if (rc) return rc;
        finish_run(e, pl, nticks);
        return SG_OK;
    }
    // The captured graph reads tick0/par0 from the segment tables uploaded by
    // prepare_run, so one graph serves every run of the same length.
    if (!e->graph_exec || e->graph_nticks != nticks || e->graph_version != e->version) {
        if (e->graph_exec) {
            cudaGraphExecDestroy(e->graph_exec);
            e->graph_exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        SG_CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_ticks(e, pl, nticks, false, true);
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return e->cuda_fail(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&e->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return e->cuda_fail(ce, "cudaGraphInstantiate");
        e->graph_nticks = nticks;
        e->graph_version = e->version;
    }
    SG_CK(cudaGraphLaunch(e->graph_exec, e->stream));
    finish_run(e, pl, nticks);
    return SG_OK;
}

int sg_engine_set_tune(sg_engine *e, const sg_tune *t)
{
    if (!e || !t) return SG_ERR_INVALID;
    if (t->blocks_per_sm < 1 || t->blocks_per_sm > 32 || t->thread_row < 1 || t->count_flavour < 0 ||
        t->count_flavour > SG_FLAVOUR_MAX)
        return e->fail(SG_ERR_INVALID, "tune parameters out of range");
    e->tune = *t;
    e->version++;
    return SG_OK;
}

int sg_last_run_active(sg_engine *e, int64_t *out, int32_t n)
{
    if (!e || (n > 0 && !out) || n < 0) return SG_ERR_INVALID;
    cudaSetDevice(e->device);
    SG_CK(cudaStreamSynchronize(e->stream));
    SgPlan pl = make_plan(e);
    if (pl.frontier) {
        if (n > e->last_nticks) return e->fail(SG_ERR_INVALID, "n exceeds the last run's ticks");
        std::vector<int32_t> len((size_t)n);
        if (n) SG_CK(cudaMemcpy(len.data(), e->flen.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
        for (int32_t r = 0; r < n; ++r) out[r] = len[(size_t)r];
        return SG_OK;
    }
    if (e->last_sweep) { // candidates of the class sweep
        if (n > e->last_nticks) return e->fail(SG_ERR_INVALID, "n exceeds the last run's ticks");
        std::vector<int32_t> c((size_t)n);
        if (n) SG_CK(cudaMemcpy(c.data(), e->tick_cand.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
        for (int32_t r = 0; r < n; ++r) out[r] = c[(size_t)r];
        return SG_OK;
    }
    int64_t agents = 0;
    for (SgStep *s : pl.order)
        if (s->kind == SG_BUILTIN_SIR_A || s->kind == SG_BUILTIN_SIR_B) agents += s->end - s->begin;
    for (int32_t r = 0; r < n; ++r) out[r] = agents;
    return SG_OK;
}

int sg_synchronize(sg_engine *e)
{
    if (!e) return SG_ERR_INVALID;
    cudaSetDevice(e->device);
    SG_CK(cudaStreamSynchronize(e->stream));
    return SG_OK;
}

int sg_snapshot(sg_engine *e)
{
    if (!e) return SG_ERR_INVALID;
    cudaSetDevice(e->device);
    for (auto &p : e->props) {
        const size_t bytes = (size_t)std::max<int64_t>(p->rows, 1) * p->row_bytes();
        SG_CK(p->snap.reserve(bytes));
        SG_CK(cudaMemcpyAsync(p->snap.p, p->buf[p->cur].p, bytes, cudaMemcpyDeviceToDevice, e->stream));
    }
    SG_CK(cudaStreamSynchronize(e->stream));
    return SG_OK;
}

int sg_restore(sg_engine *e)
{
    if (!e) return SG_ERR_INVALID;
    cudaSetDevice(e->device);
    for (auto &p : e->props) {
        if (!p->snap.p) return e->fail(SG_ERR_INVALID, "no snapshot");
        const size_t bytes = (size_t)std::max<int64_t>(p->rows, 1) * p->row_bytes();
        SG_CK(cudaMemcpyAsync(p->buf[p->cur].p, p->snap.p, bytes, cudaMemcpyDeviceToDevice, e->stream));
    }
    return SG_OK;
}

int sg_profile_enable(sg_engine *e, int32_t on)
{
    if (!e) return SG_ERR_INVALID;
    e->prof.on = on != 0;
    if (!on) {
        for (auto &k : e->prof.kinds) {
            k.launches = 0;
            k.total_ms = 0.0;
        }
    }
    return SG_OK;
}

int sg_profile_get(sg_engine *e, int32_t kind, char *name, size_t cap, int64_t *launches,
                   double *total_ms)
{
    if (!e) return SG_ERR_INVALID;
    if (kind < 0 || kind >= (int32_t)e->prof.kinds.size()) return SG_ERR_NOT_FOUND;
    const SgProfKind &k = e->prof.kinds[kind];
    if (name && cap) {
        const size_t m = std::min(cap - 1, k.name.size());
        memcpy(name, k.name.data(), m);
        name[m] = '\0';
    }
    if (launches) *launches = k.launches;
    if (total_ms) *total_ms = k.total_ms;
    return SG_OK;
}

int sg_opinion_cosine_check(sg_engine *e, int32_t k0, int32_t n, double *split, double *direct)
{
    if (!e || k0 < 0 || n < 0 || (int64_t)k0 + n > SG_BOX_MULLER_SIZE || (n > 0 && (!split || !direct)))
        return SG_ERR_INVALID;
    if (n == 0) return SG_OK;
    cudaSetDevice(e->device);
    SgDev trig, out;
    SG_CK(trig.reserve((size_t)SG_BM_TRIG_ENTRIES * sizeof(float2)));
    SG_CK(out.reserve((size_t)n * 2 * sizeof(double)));
    SG_CK(sg_launch_opinion_tables(nullptr, nullptr, trig.as<float2>(), e->stream));
    SG_CK(sg_launch_opinion_cos_check(trig.as<float2>(), k0, n, out.as<double>(), e->stream));
    std::vector<double> h((size_t)n * 2);
    SG_CK(cudaMemcpyAsync(h.data(), out.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    for (int32_t q = 0; q < n; ++q) {
        split[q] = h[2 * (size_t)q];
        direct[q] = h[2 * (size_t)q + 1];
    }
    return SG_OK;
}

int sg_opinion_noise_check(sg_engine *e, double sigma, int64_t n, const float *x, const uint32_t *k1,
                           const uint32_t *k2, float *out, float *exact, uint8_t *slow)
{
    if (!e || n < 0 || (n > 0 && (!x || !k1 || !k2 || !out || !exact || !slow))) return SG_ERR_INVALID;
    for (int64_t q = 0; q < n; ++q)
        if (k1[q] >= (uint32_t)SG_BOX_MULLER_SIZE || k2[q] >= (uint32_t)SG_BOX_MULLER_SIZE) return SG_ERR_INVALID;
    if (n == 0) return SG_OK;
    cudaSetDevice(e->device);
    SgDev radius, rq, trig, dx, dk1, dk2, dout, dexact, dslow;
    SG_CK(radius.reserve((size_t)SG_BOX_MULLER_SIZE * sizeof(float2)));
    SG_CK(rq.reserve(SG_BM_RQ_BYTES));
    SG_CK(trig.reserve((size_t)SG_BM_TRIG_ENTRIES * sizeof(float2)));
    const size_t b4 = (size_t)n * 4;
    SG_CK(dx.reserve(b4));
    SG_CK(dk1.reserve(b4));
    SG_CK(dk2.reserve(b4));
    SG_CK(dout.reserve(b4));
    SG_CK(dexact.reserve(b4));
    SG_CK(dslow.reserve((size_t)n));
    SG_CK(sg_launch_opinion_tables(radius.as<float2>(), rq.as<uint32_t>(), trig.as<float2>(), e->stream));
    SG_CK(cudaMemcpyAsync(dx.p, x, b4, cudaMemcpyHostToDevice, e->stream));
    SG_CK(cudaMemcpyAsync(dk1.p, k1, b4, cudaMemcpyHostToDevice, e->stream));
    SG_CK(cudaMemcpyAsync(dk2.p, k2, b4, cudaMemcpyHostToDevice, e->stream));
    SgTickArgs a{};
    a.bm_radius = radius.as<float2>();
    a.bm_rq = rq.as<uint32_t>();
    a.bm_trig = trig.as<float2>();
    a.sigma_hi = (float)sigma;
    a.sigma_lo = (float)(sigma - (double)a.sigma_hi);
    SG_CK(sg_launch_opinion_noise_check(a, dx.as<float>(), dk1.as<uint32_t>(), dk2.as<uint32_t>(), n,
                                        dout.as<float>(), dexact.as<float>(), (uint8_t *)dslow.p, e->stream));
    SG_CK(cudaMemcpyAsync(out, dout.p, b4, cudaMemcpyDeviceToHost, e->stream));
    SG_CK(cudaMemcpyAsync(exact, dexact.p, b4, cudaMemcpyDeviceToHost, e->stream));
    SG_CK(cudaMemcpyAsync(slow, dslow.p, (size_t)n, cudaMemcpyDeviceToHost, e->stream));
    SG_CK(cudaStreamSynchronize(e->stream));
    return SG_OK;
}

} // extern "C"
