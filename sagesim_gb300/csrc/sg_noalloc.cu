// sg_noalloc.cu -- SIR ticks for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a host application whose CUDA memory is
// owned by a pool or allocator of its own (a simulation framework embedding
// this engine, an inference server with a fixed memory plan), code running
// while a stream is being captured, or a plugin whose contract forbids
// allocation after start-up. sg_sir_run_noalloc gives them the count-strategy
// SIR tick with every piece of scratch memory it needs (the infected-neighbour
// counts, the per-tile change lists, the tile and segment tables) taken from
// one file-scope __device__ array of fixed size, SG_NOALLOC_SCRATCH_BYTES,
// which every GPU that loads this library holds until the process exits. The
// caller passes the CSR and the state array (device pointers) and gets the
// state back in place.
//
// The array is shared by every call: two calls whose work overlaps on the GPU
// (different streams, no ordering between them) race on it and give wrong
// results. Calls issued on one stream, or otherwise ordered, are safe; each
// call clears the part of the array it reads before reading it.
#include <cuda.h> // CUcontext / CUresult types only; the calls go through entry points
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/sagesim_gb300.h"
#include "sg_kernels.h"
#include "sg_philox.h"

void sg_set_thread_error(const std::string &msg); // sg_engine.cu

namespace {

constexpr int64_t kMaxAgents = SG_NOALLOC_MAX_AGENTS;
constexpr int64_t kMaxTiles = (kMaxAgents + SG_TILE - 1) / SG_TILE;

// layout of the scratch array (byte offsets, each 256-byte aligned)
constexpr size_t kCntOff = 0;
constexpr size_t kChangesOff = kCntOff + (size_t)kMaxAgents * 4;
constexpr size_t kTileNchOff = kChangesOff + (size_t)kMaxAgents * 4;
constexpr size_t kTilesOff = kTileNchOff + ((size_t)kMaxTiles * 4 + 255) / 256 * 256;
constexpr size_t kSegOff = kTilesOff + ((size_t)kMaxTiles * sizeof(SgTile) + 255) / 256 * 256;
constexpr size_t kEnd = kSegOff + (sizeof(SgSeg) + 255) / 256 * 256;
static_assert(kEnd <= SG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[SG_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per CUDA context. In host code the
// symbol name is only a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress once per context, with that context's device current,
// and handed to the kernels. The cache is keyed on the context's unique id
// (cuCtxGetId), not on the device number: after cudaDeviceReset, or with a
// non-primary context current, the id differs and the address is looked up
// again instead of reusing one that belongs to another (or a destroyed)
// context. The two driver calls are reached through the runtime's
// driver-entry-point lookup, so the library still links no driver library.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

std::mutex g_mu;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
std::vector<std::pair<unsigned long long, void *>> g_scratch; // context id -> device address

int noalloc_fail(const char *what, cudaError_t ce)
{
    sg_set_thread_error(std::string("sg_sir_run_noalloc: ") + what + ": " + cudaGetErrorString(ce));
    return SG_ERR_CUDA;
}

// Id of the current context; 0 when none is current yet. Called with g_mu held.
int current_context_id(unsigned long long *id)
{
    *id = 0;
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        cudaError_t ce = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void **)&g_ctx_get_current, 12000,
                                                          cudaEnableDefault, &q1);
        if (ce == cudaSuccess)
            ce = cudaGetDriverEntryPointByVersion("cuCtxGetId", (void **)&g_ctx_get_id, 12000, cudaEnableDefault,
                                                  &q2);
        if (ce != cudaSuccess || q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess ||
            !g_ctx_get_current || !g_ctx_get_id) {
            g_ctx_get_current = nullptr;
            g_ctx_get_id = nullptr;
            return noalloc_fail("driver entry points cuCtxGetCurrent / cuCtxGetId", ce);
        }
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return noalloc_fail("cuCtxGetCurrent", cudaErrorUnknown);
    if (!ctx) return SG_OK;
    if (g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return noalloc_fail("cuCtxGetId", cudaErrorUnknown);
    return SG_OK;
}

int scratch_for_current_context(void **out)
{
    int dev = -1;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess || dev < 0) return noalloc_fail("cudaGetDevice", ce);
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc) return rc;
    if (id)
        for (const auto &e : g_scratch)
            if (e.first == id) {
                *out = e.second;
                return SG_OK;
            }
    // first call in this context (or no context current yet: the lookup makes
    // the device's primary context current)
    void *p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess || !p) return noalloc_fail("cudaGetSymbolAddress", ce);
    if (!id) {
        rc = current_context_id(&id);
        if (rc) return rc;
    }
    if (id) g_scratch.emplace_back(id, p);
    *out = p;
    return SG_OK;
}

// Writes the segment record and the tile list into the scratch array (kernel
// arguments carry the values, so no host-to-device copy is needed).
__global__ void noalloc_tables_kernel(SgSeg seg, SgSeg *dseg, SgTile *tiles, int32_t n, int32_t ntiles)
{
    const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) *dseg = seg;
    if (t < ntiles) {
        const int32_t b = t * SG_TILE;
        const int32_t e = b + SG_TILE < n ? b + SG_TILE : n;
        tiles[t] = SgTile{0, b, e, 0};
    }
}

} // namespace

extern "C" int sg_sir_run_noalloc(const int32_t *d_offsets, const int32_t *d_indices, int32_t *d_state,
                                  int64_t n, int32_t builtin, int64_t seed, int64_t tick0,
                                  int32_t nticks, double beta, double gamma, int32_t code_s,
                                  int32_t code_i, int32_t code_r, void *stream)
{
    if (n < 0 || n > kMaxAgents) {
        sg_set_thread_error("sg_sir_run_noalloc: n = " + std::to_string((long long)n) +
                            " agents is outside [0, SG_NOALLOC_MAX_AGENTS = " +
                            std::to_string((long long)kMaxAgents) + "]; use the engine API");
        return SG_ERR_INVALID;
    }
    if (builtin != SG_BUILTIN_SIR_A && builtin != SG_BUILTIN_SIR_B) {
        sg_set_thread_error("sg_sir_run_noalloc: builtin must be SG_BUILTIN_SIR_A or SG_BUILTIN_SIR_B");
        return SG_ERR_INVALID;
    }
    if (nticks < 0) {
        sg_set_thread_error("sg_sir_run_noalloc: nticks < 0");
        return SG_ERR_INVALID;
    }
    if (n == 0 || nticks == 0) return SG_OK;
    if (!d_offsets || !d_indices || !d_state) {
        sg_set_thread_error("sg_sir_run_noalloc: NULL device pointer");
        return SG_ERR_INVALID;
    }
    void *base = nullptr;
    int rc = scratch_for_current_context(&base);
    if (rc != SG_OK) return rc;
    unsigned char *b = static_cast<unsigned char *>(base);
    cudaStream_t st = (cudaStream_t)stream;
    const int32_t ntiles = (int32_t)((n + SG_TILE - 1) / SG_TILE);

    SgSeg seg{};
    seg.tick0 = tick0;
    seg.end_tick = INT64_MAX;
    seg.lids = nullptr; // RNG key = agent index
    seg.lid_base = 0;
    seg.variant = builtin;
    seg.key = (uint32_t)(uint64_t)seed;
    seg.kinf = sg_threshold_host(beta);
    seg.krec = sg_threshold_host(gamma);
    seg.cs = code_s;
    seg.ci = code_i;
    seg.cr = code_r;
    seg.par0 = 0;
    seg.stats = nullptr;

    SgSeg *dseg = reinterpret_cast<SgSeg *>(b + kSegOff);
    SgTile *dtiles = reinterpret_cast<SgTile *>(b + kTilesOff);
    int32_t *cnt = reinterpret_cast<int32_t *>(b + kCntOff);
    cudaError_t ce = cudaMemsetAsync(cnt, 0, (size_t)n * 4, st);
    if (ce == cudaSuccess) {
        noalloc_tables_kernel<<<(ntiles + 255) / 256, 256, 0, st>>>(seg, dseg, dtiles, (int32_t)n, ntiles);
        ce = cudaGetLastError();
    }
    int sms = 0;
    if (ce == cudaSuccess) {
        int dev = 0;
        ce = cudaGetDevice(&dev);
        if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (ce == cudaSuccess && sms <= 0) ce = cudaErrorInvalidDevice;
    }
    SgTickArgs a{};
    a.off = d_offsets;
    a.idx = d_indices;
    a.buf0 = d_state; // state updated in place
    a.buf1 = d_state;
    a.segs = dseg;
    a.tiles = dtiles;
    a.ntiles = ntiles;
    a.cnt = cnt;
    a.changes = reinterpret_cast<int32_t *>(b + kChangesOff);
    a.tile_nch = reinterpret_cast<int32_t *>(b + kTileNchOff);
    a.toff = d_offsets; // undirected graph: the CSR is its own transpose
    a.tidx = d_indices;
    a.mega = nullptr;
    a.nmega = 0;
    a.mega_blocks = 0;
    a.mega_row = INT32_MAX; // every long row goes through the warp path
    const int grid = ntiles < sms * 8 ? ntiles : sms * 8;
    if (ce == cudaSuccess) ce = sg_launch_sir_count_init(a, grid, st);
    for (int32_t r = 0; r < nticks && ce == cudaSuccess; ++r) {
        a.r = r;
        ce = sg_launch_sir_count_step(a, builtin == SG_BUILTIN_SIR_A ? 1 : 2, false, true, grid, st);
        if (ce == cudaSuccess) ce = sg_launch_sir_count_scatter(a, sms * 4, st);
    }
    if (ce != cudaSuccess) {
        sg_set_thread_error(std::string("sg_sir_run_noalloc: ") + cudaGetErrorString(ce));
        return SG_ERR_CUDA;
    }
    return SG_OK;
}
