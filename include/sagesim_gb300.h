/*
 * sagesim_gb300.h -- C ABI of the GB300 engine for SAGESim's per-tick agent step.
 *
 * Conventions
 *   - Every function returns an int status: SG_OK (0) or one of SG_ERR_*.
 *     sg_last_error() gives the message of the last failure on a handle.
 *   - Handles are opaque. The caller owns every host array it passes; the
 *     engine copies what it keeps. The engine owns all device memory it
 *     allocates and frees it in the matching *_destroy call.
 *   - A handle is not thread-safe; one handle issues work on one CUDA stream
 *     (the caller's, if given in sg_engine_cfg.stream, else its own).
 *   - Agent indices and CSR offsets are int32: an engine holds fewer than
 *     2^31 agents and 2^31 CSR entries.
 *   - Philox draws are keyed exactly as SAGESim keys them
 *     (sagesim/math_utils.py:106-189): counter (tick*1000003 + salt, logical id),
 *     key = seed, all mod 2^32; u = (c0 mod 2^23) / 2^23.
 *
 * Reference interfaces replaced (file:line in the SAGESim source tree):
 *   sg_engine_create/destroy      Model.__init__ / reset()      sagesim/model.py:357-386, 944-958
 *   sg_set_graph_csr              NetworkSpace adjacency -> CSR sagesim/space.py:107-125,
 *                                                               sagesim/internal_utils.py:111-186,
 *                                                               sagesim/model.py:1143-1148
 *   sg_set_graph_id_edges         convert_agent_ids_to_indices  sagesim/model.py:31-110,
 *                                 + CSR build (on the GPU)      sagesim/model.py:1068-1148
 *   sg_set_logical_ids            set_agent_logical_id          sagesim/model.py:656-667, 1089-1096
 *   sg_set_seed                   set_seed                      sagesim/model.py:652-654
 *   sg_set_globals_f64            register/set_global_property  sagesim/model.py:588-604
 *   sg_add_property               Breed.register_property +
 *                                 property tensor upload        sagesim/breed.py:40-61,
 *                                                               sagesim/model.py:1192-1197
 *   sg_add_array                  register_breed_local_array +  sagesim/model.py:620-650,
 *                                 breed-local array build       sagesim/model.py:1215-1270
 *   sg_set_property/get_property  set/get_agent_property_value,
 *                                 get_breed_data                sagesim/model.py:422-490
 *   sg_add_builtin_step           register_step_func (builtin)  sagesim/breed.py:68-99
 *   sg_compile_step               register_step_func + codegen  sagesim/breed.py:68-99,
 *                                                               sagesim/model.py:2010-2457
 *   sg_run                        simulate -> worker_coroutine  sagesim/model.py:961-998, 1314-1640
 *   sg_get_tick_history           per-tick S/I/R/E_S dumps      (no counterpart; the reference's
 *                                                               tests read agents one by one,
 *                                                               sagesim/model.py:422-450)
 */
#ifndef SAGESIM_GB300_H
#define SAGESIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define SG_OK 0
#define SG_ERR_INVALID 1   /* bad argument or call order                      */
#define SG_ERR_BAD_CSR 2   /* offsets not monotone / index out of range       */
#define SG_ERR_CUDA 3      /* a CUDA runtime call failed                      */
#define SG_ERR_OOM 4       /* device allocation failed                        */
#define SG_ERR_COMPILE 5   /* NVRTC rejected a step source (log in message)   */
#define SG_ERR_BUDGET 6    /* request larger than the server's HBM budget     */
#define SG_ERR_TIMEOUT 7   /* a bounded device-side wait gave up              */
#define SG_ERR_OOB 8       /* a device bounds check fired (checked builds)    */
#define SG_ERR_NOT_FOUND 9 /* unknown id                                      */

/* ---- dtypes ------------------------------------------------------------ */
#define SG_I32 0
#define SG_F32 1

/* ---- builtin steps ------------------------------------------------------ */
/* SIR with one draw per agent per tick (SAGESim's own test step,
 * tests/test_simulation.py:24-43). */
#define SG_BUILTIN_SIR_A 1
/* SIR with one Bernoulli(beta) trial per infected neighbour (salts 2, 3, ...). */
#define SG_BUILTIN_SIR_B 2
/* Opinion update: weighted mean of the first `width` ordered neighbours plus
 * Philox N(0, sigma) noise, clamped to [0, 1]. */
#define SG_BUILTIN_OPINION 3

/* ---- SIR evaluation strategy (same results, different work) ---------------- */
/* Pull: each susceptible agent scans its CSR row every tick (degree-binned:
 * thread per agent, warp per hub). */
#define SG_SIR_PULL 0
/* Count: the engine keeps, per agent, the number of infected neighbours and
 * updates it only for agents whose state changed (needs the transpose CSR,
 * built once per graph). */
#define SG_SIR_COUNT 1
/* Frontier: like count, but each tick touches only the active agents
 * (infected, or susceptible with an infected neighbour), kept in a compact
 * list; the SIR step must be the engine's only step (state updated in place). */
#define SG_SIR_FRONTIER 2

/* ---- graph flags ------------------------------------------------------------ */
/* Row order matters (NetworkSpace(ordered=True), sagesim/space.py:54-71). */
#define SG_GRAPH_ORDERED 1
/* The caller asserts the CSR is symmetric (undirected graph); the count
 * strategy then reuses it as its own transpose. */
#define SG_GRAPH_SYMMETRIC 2

typedef struct sg_engine sg_engine;

typedef struct sg_engine_cfg {
    int32_t device;  /* CUDA device ordinal                                   */
    int32_t flags;   /* reserved, 0                                           */
    void *stream;    /* cudaStream_t to issue work on; NULL = engine-owned     */
} sg_engine_cfg;

/* Parameters of a builtin step. Probabilities are float64 like SAGESim globals
 * (sagesim/model.py:593); the kernel compares the 23-bit Philox integer against
 * the exact integer threshold ceil(p * 2^23), which is the same test as the
 * reference's double compare `u < p`. */
typedef struct sg_builtin_params {
    int32_t builtin;        /* SG_BUILTIN_*                                          */
    int32_t strategy;       /* SIR: SG_SIR_PULL or SG_SIR_COUNT                       */
    int32_t state_prop;     /* SIR: int32 state property; OPINION: float32 opinion    */
    int32_t aux_prop;       /* OPINION: float32[width] weights property; else -1      */
    int32_t code_s, code_i, code_r; /* SIR state codes (SAGESim tests use 1, 2, 3)  */
    int32_t priority;       /* execution priority (lower runs first)                  */
    int64_t begin, end;     /* agent range the step runs over (a breed's range)       */
    double beta, gamma;     /* SIR probabilities                                      */
    double sigma;           /* OPINION noise standard deviation                       */
} sg_builtin_params;

/* Per-run statistics. */
typedef struct sg_stats {
    int64_t ticks;          /* ticks executed                                   */
    int64_t agent_ticks;    /* agents x ticks over the stepped ranges           */
    int64_t edge_visits;    /* sum over ticks of E_S (degree sum of the agents
                               susceptible at tick start); SIR only             */
    double device_ms;       /* device time of the run (CUDA events)             */
    int64_t kernel_launches; /* kernels the run launched                        */
} sg_stats;

/* Launch configuration the autotuner chooses between (all give identical results). */
typedef struct sg_tune {
    int32_t strategy;          /* SG_SIR_PULL or SG_SIR_COUNT                     */
    int32_t blocks_per_sm;     /* persistent grid = blocks_per_sm x SM count     */
    int32_t thread_row;        /* rows up to this length: one lane; longer: warp */
    int32_t mega_row;          /* rows longer than this: a whole block           */
    int32_t count_flavour;     /* count strategy, bit mask (0..1023):            */
                               /*  1 = 8 agents per thread (else 4)              */
                               /*  2 = warp-dense SIR-B draws                    */
                               /*  4 = count and RNG key loaded only where needed*/
                               /*  8 = scatter: one transpose row per lane       */
                               /* 16 = class sweep (in-place runs, graphs of at  */
                               /*      least 2 tiles of 2048 agents per SM)      */
                               /* 32 = class sweep on graphs of any size         */
                               /* bits 6-7: sweep warps per tile, 0 = automatic, */
                               /*      1/2/3 = 1/2/4 warps                       */
                               /* 256 = with 16: hybrid, the loop form of bits   */
                               /*      0-2 in busy ticks (decided on the GPU;    */
                               /*      graphs of 24+ tiles per SM, or with 32)   */
                               /* 512 = flat draws in place of the loop form     */
                               /*      (in-place runs): a warp lays its agents'  */
                               /*      draws end to end, each lane an equal      */
                               /*      share                                     */
                               /* default 790: class sweep + hybrid whose busy-  */
                               /*      tick form is the flat draws, both in one  */
                               /*      launch per tick (the loop form's bits 2   */
                               /*      and 4 apply where flat draws cannot run:  */
                               /*      runs not in place)                        */
    double us_per_tick;        /* measured by sg_batch_tune (output)             */
} sg_tune;

/* ---- engine lifecycle ------------------------------------------------------- */
int sg_engine_create(const sg_engine_cfg *cfg, sg_engine **out);
int sg_engine_destroy(sg_engine *e);
/* Copies the last error message of `e` (or of the last failed create when e is
 * NULL) into buf (always NUL-terminated when cap > 0). */
int sg_last_error(const sg_engine *e, char *buf, size_t cap);

/* ---- model definition -------------------------------------------------------- */
/* CSR of the agent graph: agent i's neighbours are indices[offsets[i] ..
 * offsets[i+1]). Validates offsets[0] == 0, monotone offsets, offsets[n] == nnz
 * and every index in [0, n); SG_ERR_BAD_CSR otherwise. Replaces any previous
 * graph and fixes the agent count n; once properties exist it may be called
 * between runs with the same n (topology edits, sagesim/space.py:107-145): the
 * next run rebuilds its tile tables and counts from the new graph. */
int sg_set_graph_csr(sg_engine *e, const int32_t *offsets, int64_t n, const int32_t *indices,
                     int64_t nnz, int32_t flags);
/* Graph from an edge list in agent ids, built on the GPU (replaces the
 * reference's id -> index conversion, sagesim/model.py:31-110, and its host CSR
 * build, sagesim/internal_utils.py:111-186, for NetworkSpace.connect_agents
 * graphs). ids[0..n): each agent's id in buffer order (distinct, any int64 but
 * INT64_MIN); an open-addressing hash table in HBM maps ids to buffer indices.
 * (src_ids[k], dst_ids[k]), k < nedges: host arrays of edges. flags:
 * SG_GRAPH_SYMMETRIC adds each edge in both directions; SG_GRAPH_ORDERED keeps
 * a row in first-connection order (NetworkSpace(ordered=True)), else rows are
 * sorted by neighbour index. Repeated edges are dropped. A repeated id is
 * SG_ERR_INVALID, an edge naming an unknown id SG_ERR_BAD_CSR. */
int sg_set_graph_id_edges(sg_engine *e, const int64_t *ids, int64_t n, const int64_t *src_ids,
                          const int64_t *dst_ids, int64_t nedges, int32_t flags);
/* Copies the engine's CSR to host arrays (offsets: n + 1, indices: nnz; either
 * may be NULL) and returns nnz. */
int sg_get_graph_csr(sg_engine *e, int32_t *offsets, int32_t *indices, int64_t *nnz);
/* RNG key per agent (default: the agent index). */
int sg_set_logical_ids(sg_engine *e, const int64_t *lids, int64_t n);
int sg_set_seed(sg_engine *e, int64_t seed);
/* Global parameters visible to compiled step functions as `const double* g`. */
int sg_set_globals_f64(sg_engine *e, const double *values, int32_t n);
/* Adds a per-agent property of `width` values of `dtype`; init holds n*width
 * values (NULL = zeros). `double_buffered` = 0 writes in place (SAGESim's
 * no_double_buffer, sagesim/breed.py:68-99). */
int sg_add_property(sg_engine *e, const char *name, int32_t dtype, int32_t width,
                    int32_t double_buffered, const void *init, int32_t *prop_id);
/* Adds a breed-local array (Model.register_breed_local_array,
 * sagesim/model.py:620-650, storage built at sagesim/model.py:1215-1270):
 * `rows` rows of `width` values of `dtype`, init holds rows*width values (NULL =
 * zeros). It is a property whose row count is not the agent count: steps read
 * and write it through the same property table (ctx.arr_f32 / set_arr_f32),
 * double-buffered unless double_buffered = 0, and sg_set_property /
 * sg_get_property / snapshots address its rows. */
int sg_add_array(sg_engine *e, const char *name, int32_t dtype, int32_t width, int64_t rows,
                 int32_t double_buffered, const void *init, int32_t *prop_id);
/* Host <-> device copies of rows [first, first+count) of a property (agents) or
 * an array. */
int sg_set_property(sg_engine *e, int32_t prop, const void *host, int64_t first, int64_t count);
int sg_get_property(sg_engine *e, int32_t prop, void *host, int64_t first, int64_t count);
/* Device pointer of a property's current (read) buffer, for zero-copy callers. */
int sg_property_device_ptr(sg_engine *e, int32_t prop, void **dptr);

/* ---- steps --------------------------------------------------------------------- */
int sg_add_builtin_step(sg_engine *e, const sg_builtin_params *p, int32_t *step_id);
/* Replaces the parameters of a builtin step (same builtin and state property),
 * e.g. after set_global_property_value (sagesim/model.py:599-604). */
int sg_update_builtin_step(sg_engine *e, int32_t step_id, const sg_builtin_params *p);
/* Compiles a CUDA C++ step with NVRTC and adds it at `priority` over agents
 * [begin, end). `cuda_src` defines
 *   __device__ void <entry>(const sg_ctx& ctx, int i)
 * (sg_ctx is in sagesim_gb300_step.h, included automatically). written_props
 * lists the properties the step writes. SG_ERR_COMPILE carries the NVRTC log. */
int sg_compile_step(sg_engine *e, const char *cuda_src, const char *entry, int32_t priority,
                    int64_t begin, int64_t end, const int32_t *written_props, int32_t n_written,
                    int32_t *step_id);

/* ---- execution ------------------------------------------------------------------ */
/* Runs ticks [tick0, tick0 + nticks): per tick every priority in order, reads of
 * double-buffered properties seeing tick-start values, then the write-back.
 * tick_stats (nullable, host): 4 int64 per tick = S, I, R after the tick and E_S,
 * summed over the SIR steps. out (nullable) gets totals. Synchronous. */
int sg_run(sg_engine *e, int64_t tick0, int32_t nticks, int64_t *tick_stats, sg_stats *out);
/* Per-tick history for parity dumps: the S, I, R, E_S rows (as in tick_stats)
 * of consecutive sg_run calls that took statistics, from the tick *first_tick
 * on; a run that does not continue them starts a new history. Copies up to
 * max_ticks rows into out (nullable) and returns the row count in *nticks. */
int sg_get_tick_history(sg_engine *e, int64_t *out, int64_t max_ticks, int64_t *nticks, int64_t *first_tick);
/* Same, asynchronous on the engine stream: returns after enqueueing (through a
 * CUDA graph of the tick loop when use_graph != 0). No stats. */
int sg_run_async(sg_engine *e, int64_t tick0, int32_t nticks, int32_t use_graph);
int sg_synchronize(sg_engine *e);

/* Launch configuration of the engine's SIR kernels (strategy is ignored: it is
 * a property of the step). All configurations give identical results. */
int sg_engine_set_tune(sg_engine *e, const sg_tune *t);

/* Agents the SIR step processed in each tick of the last sg_run/sg_run_async
 * (the active list length for the frontier strategy; the candidates -- infected
 * agents and susceptible agents whose activity bit is set -- for the class
 * sweep; the step's agent range otherwise); n = number of ticks to report.
 * Synchronizes the stream. */
int sg_last_run_active(sg_engine *e, int64_t *out, int32_t n);

/* Device snapshot of every property (checkpoint in HBM) and restore. */
int sg_snapshot(sg_engine *e);
int sg_restore(sg_engine *e);

/* Profiling: when enabled, sg_run brackets every kernel launch with CUDA events
 * and accumulates time per kernel kind. */
int sg_profile_enable(sg_engine *e, int32_t on);
/* kind index -> name, launch count, total milliseconds; SG_ERR_NOT_FOUND past the end. */
int sg_profile_get(sg_engine *e, int32_t kind, char *name, size_t cap, int64_t *launches,
                   double *total_ms);

/* The opinion step's cosine cos(2 pi k / 2^23) (the Box-Muller angle of
 * sagesim/math_utils.py:250-255) as the step forms it from its split tables,
 * split[q], and evaluated directly with the device's cos, direct[q], for
 * k = k0 .. k0 + n - 1 (k0 + n <= 2^23). A check of the engine's own table
 * method; no counterpart in the reference. */
int sg_opinion_cosine_check(sg_engine *e, int32_t k0, int32_t n, double *split, double *direct);

/* The opinion step's noise term for n host triples (opinion x[q], the normal
 * draw's 23-bit integers k1[q], k2[q] < 2^23) at noise level sigma:
 * out[q] = clamp(float32(x + sigma * sqrt(-2 log(k1 / 2^23 + 1e-10)) *
 * cos(2 pi k2 / 2^23)), 0, 1) exactly as the step forms it (fixed-point radius,
 * the pair table where the rounding is open), exact[q] = the same with the
 * pair-table radius always, slow[q] = 1 where the pair table was needed. A
 * check of the engine's own table method; no counterpart in the reference.
 * SG_ERR_INVALID for a k outside [0, 2^23) or NULL arrays with n > 0. */
int sg_opinion_noise_check(sg_engine *e, double sigma, int64_t n, const float *x, const uint32_t *k1,
                           const uint32_t *k2, float *out, float *exact, uint8_t *slow);

/* ---- ensembles: many independent SIR scenarios in one launch per tick ---------------
 * No single counterpart in the reference, which runs one model per process
 * (sagesim/model.py:961-998); each scenario here is what one reference Model
 * with one SIR breed would simulate, and stays bit-exact with its standalone
 * run: it keeps its own seed, logical ids, tick counter (starting at 0) and
 * horizon. Scenarios are packed into one device pool (global CSR, state,
 * segment table, tile list); every kernel launch advances all of them. The
 * tick loop of sg_batch_run is captured once as a CUDA graph and replayed. */
typedef struct sg_batch sg_batch;

typedef struct sg_scenario_desc {
    int64_t n_agents;          /* agents of the scenario                                   */
    int64_t nnz;               /* CSR entries                                              */
    const int32_t *offsets;    /* host CSR (local indices), copied                         */
    const int32_t *indices;
    const int32_t *state;      /* host initial state, n_agents int32                      */
    const int64_t *lids;       /* host RNG keys or NULL (= local agent index)              */
    int64_t seed;
    double beta, gamma;
    int32_t builtin;           /* SG_BUILTIN_SIR_A or SG_BUILTIN_SIR_B (same for a batch)  */
    int32_t code_s, code_i, code_r;
    int32_t horizon;           /* ticks the scenario runs; later ticks skip it             */
    int32_t flags;             /* SG_GRAPH_SYMMETRIC when the CSR is its own transpose     */
} sg_scenario_desc;


int sg_batch_create(const sg_engine_cfg *cfg, sg_batch **out);
int sg_batch_destroy(sg_batch *b);
int sg_batch_last_error(const sg_batch *b, char *buf, size_t cap);
/* Stages a scenario (host copy); returns its id. Validates the CSR. */
int sg_batch_add_scenario(sg_batch *b, const sg_scenario_desc *d, int32_t *sid);
/* Packs the staged scenarios into the device pool (once, before running). */
int sg_batch_commit(sg_batch *b);
int sg_batch_set_tune(sg_batch *b, const sg_tune *t);
int sg_batch_get_tune(sg_batch *b, sg_tune *t);
/* Times every candidate launch configuration on `ticks` ticks from the
 * current state (restored afterwards), keeps the fastest and returns it. */
int sg_batch_tune(sg_batch *b, int32_t ticks, sg_tune *best);
/* Advances every scenario by up to nticks ticks (none past its horizon).
 * use_graph: replay a captured CUDA graph of the tick loop. Asynchronous. */
int sg_batch_run(sg_batch *b, int32_t nticks, int32_t use_graph);
int sg_batch_synchronize(sg_batch *b);
/* Current state of a scenario (host copy, synchronous) and its tick count. */
int sg_batch_get_state(sg_batch *b, int32_t sid, int32_t *host, int64_t n);
int sg_batch_scenario_tick(sg_batch *b, int32_t sid, int64_t *tick);
/* Totals of the batch: agents, CSR entries, device bytes held. */
int sg_batch_info(sg_batch *b, int64_t *agents, int64_t *nnz, int64_t *device_bytes);
/* Device snapshot of the state of every scenario (and its tick) and restore. */
int sg_batch_snapshot(sg_batch *b);
int sg_batch_restore(sg_batch *b);

/* ---- serving: continuous batching of scenario requests ----------------------------------
 * No counterpart in the reference. Requests (one SIR scenario each, with its
 * own horizon) are admitted FIFO against an HBM budget and the free space of a
 * resident scenario pool; every sg_server_step admits what fits, advances all
 * resident scenarios together by nticks (one CUDA-graph replay), and retires
 * the ones that reached their horizon, whose final state is kept on the host
 * until taken. A request never sees another's data: each result equals the
 * scenario's standalone run. A request larger than the whole budget or pool is
 * refused at submission with SG_ERR_BUDGET. A request passed over 8 times by
 * smaller ones that fitted stops later requests from being admitted ahead of it. */
typedef struct sg_server sg_server;

typedef struct sg_server_cfg {
    int32_t device;
    int32_t builtin;         /* SIR variant of every request                       */
    void *stream;            /* NULL = server-owned stream                         */
    int64_t budget_bytes;    /* admission budget for resident scenarios            */
    int64_t agent_slots;     /* device pool capacity: agents (+1 per scenario)      */
    int64_t edge_slots;      /* device pool capacity: CSR entries                   */
    int32_t max_resident;    /* scenarios resident at once                          */
    int32_t flags;           /* reserved, 0                                         */
} sg_server_cfg;

#define SG_REQ_QUEUED 0
#define SG_REQ_RUNNING 1
#define SG_REQ_DONE 2
/* A borrowed request whose CSR the device check refused when it was placed;
 * sg_server_take_result then returns SG_ERR_BAD_CSR and forgets it. */
#define SG_REQ_FAILED 3
/* sg_scenario_desc.flags for sg_server_submit: the caller keeps offsets,
 * indices, state and lids valid and unchanged until the request has left the
 * queue (poll status other than SG_REQ_QUEUED). A queued request then keeps
 * the pointers instead of host copies, and its CSR is checked on the device
 * when it is placed (no host pass over the edges at submission). */
#define SG_REQ_BORROW 256

int sg_server_create(const sg_server_cfg *cfg, sg_server **out);
int sg_server_destroy(sg_server *s);
int sg_server_last_error(const sg_server *s, char *buf, size_t cap);
/* Submits a request; the CSR must be symmetric. d->lids (nullable) gives each
 * agent's logical id, the key of its draws (sagesim/model.py:656-667), so a
 * request relabelled for locality reproduces its run in the original order.
 * With nothing queued and room in the budget and pool it is placed on the
 * device at once (status RUNNING; the CSR is checked there), else queued (the
 * host arrays are checked and copied). Either way the caller's arrays are free
 * again when the call returns. */
int sg_server_submit(sg_server *s, const sg_scenario_desc *d, int64_t *rid);
/* Admits, runs nticks for every resident scenario, retires the finished ones.
 * Synchronous. n_done (nullable) = requests finished by this step. */
int sg_server_step(sg_server *s, int32_t nticks, int32_t *n_done);
/* status = SG_REQ_*; tick = ticks done so far. */
int sg_server_poll(sg_server *s, int64_t rid, int32_t *status, int64_t *tick);
/* Copies a finished request's final state and forgets the request. */
int sg_server_take_result(sg_server *s, int64_t rid, int32_t *host, int64_t n);
int sg_server_counts(sg_server *s, int64_t *queued, int64_t *resident, int64_t *done,
                     int64_t *resident_bytes);
/* Sets the launch configuration of the resident pool (see sg_tune). */
int sg_server_set_tune(sg_server *s, const sg_tune *t);

/* ---- allocation-free SIR ticks ------------------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory (their memory is owned by a pool or plan of their own, they run while
 * a stream is captured, or their plugin contract forbids allocation): runs
 * nticks ticks [tick0, tick0 + nticks) of SIR (builtin = SG_BUILTIN_SIR_A or
 * SG_BUILTIN_SIR_B, count strategy) on an undirected graph given as a
 * symmetric CSR in device memory, updating d_state (int32, device) in place,
 * RNG key = agent index. All scratch memory comes from one static device array
 * of SG_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * exit; the call allocates nothing. n above SG_NOALLOC_MAX_AGENTS is rejected
 * with SG_ERR_INVALID (message via sg_last_error(NULL, ...)). The first call in
 * each CUDA context (the device's primary context, again after a device reset,
 * or a context of the caller's own) looks up the array's device address
 * (cudaGetSymbolAddress) with that context current; make that first call before
 * any stream capture. Calls
 * share the array: calls that overlap on the GPU race and give wrong results;
 * calls on one stream are safe. Asynchronous on `stream` (NULL = legacy). */
#define SG_NOALLOC_MAX_AGENTS 1048576
#define SG_NOALLOC_SCRATCH_BYTES (8u * 1048576u + 16384u)
int sg_sir_run_noalloc(const int32_t *d_offsets, const int32_t *d_indices, int32_t *d_state,
                       int64_t n, int32_t builtin, int64_t seed, int64_t tick0, int32_t nticks,
                       double beta, double gamma, int32_t code_s, int32_t code_i, int32_t code_r,
                       void *stream);

/* ---- host-side workload utilities (no counterpart in the reference, which
 * builds graphs with networkx and partitions with METIS:
 * sagesim/generate_partition.py:24-69, sagesim/partition_utils.py:39-103) ---- */
/* Undirected graphs as symmetric CSR without self loops or duplicate edges.
 * Two-pass: call with offsets/indices NULL to get nnz, then with buffers. */
int sg_graph_er(int64_t n, double p, uint64_t seed, int32_t *offsets, int32_t *indices,
                int64_t *nnz);
int sg_graph_ba(int64_t n, int32_t m, uint64_t seed, int32_t *offsets, int32_t *indices,
                int64_t *nnz);
/* Watts-Strogatz ring lattice (k neighbours) with rewiring probability p; rows
 * list neighbours in edge-insertion order (NetworkSpace(ordered=True)). */
int sg_graph_ws(int64_t n, int32_t k, double p, uint64_t seed, int32_t *offsets,
                int32_t *indices, int64_t *nnz);
/* Seeded k-way locality partition (graph growing from k seeds, balanced parts,
 * BFS order inside a part). perm[old] = new index; part[new] (nullable) = part id. */
int sg_partition_relabel(int64_t n, const int32_t *offsets, const int32_t *indices, int32_t k,
                         uint64_t seed, int32_t *perm, int32_t *part);
/* Applies perm (perm[old] = new) to a CSR: row new = perm[old] lists perm[nbr]
 * in the original order. */
int sg_csr_permute(int64_t n, const int32_t *offsets, const int32_t *indices,
                   const int32_t *perm, int32_t *new_offsets, int32_t *new_indices);

#ifdef __cplusplus
}
#endif
#endif /* SAGESIM_GB300_H */
