// sg_kernels.h -- launch interface of the tick kernels (host side).
//
// All tick kernels walk a tile list: a tile is a range of consecutive agents
// that belong to one segment (one SIR/opinion step over one scenario's agent
// range). A plain engine has one segment; an ensemble batch has one segment per
// scenario. Tick-invariant per-segment data lives in a device table; the only
// per-tick kernel argument is r, the tick index relative to the start of the
// run, so a captured CUDA graph of the tick loop needs no host updates.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define SG_TILE 2048       // agents per tile
#define SG_SIR_THREADS 256 // threads per block of the tick kernels

struct SgSeg {
    int64_t tick0;          // segment's absolute tick at r == 0
    int64_t end_tick;       // the segment does no work at ticks >= end_tick
    const uint32_t *lids;   // RNG key (lid mod 2^32) per global agent index; NULL -> i - lid_base
    int32_t lid_base;       // global index of the segment's first agent
    int32_t variant;        // 1 = SIR-A, 2 = SIR-B, 3 = opinion
    uint32_t key;           // seed mod 2^32
    uint32_t kinf, krec;    // integer thresholds (SIR)
    int32_t cs, ci, cr;     // SIR state codes
    int32_t par0;           // state at tick0 lives in buffer [par0] of the pair
    int32_t width;          // opinion: weights per agent
    double sigma;           // opinion: noise standard deviation
    unsigned long long *stats; // NULL or [ticks][4] counters, row r
    const float *weights;   // opinion: [n][width] (global agent index)
};

struct SgTile {
    int32_t seg, begin, end, pad;
};

// An agent whose CSR row is longer than SgTickArgs::mega_row; scanned by a
// whole block (listed once per graph).
struct SgMega {
    int32_t agent, seg;
};

// Count-step flavours (bit mask; every flavour gives the same result).
#define SG_FLAVOUR_PER8 1   // 8 agents per thread and pass instead of 4
#define SG_FLAVOUR_DENSE 2  // warp-dense SIR-B draws
#define SG_FLAVOUR_LAZY 4   // count and RNG key loaded only where needed
#define SG_FLAVOUR_ROWSCATTER 8 // scatter walks one transpose row per lane instead of
                                // the warp's rows laid end to end
#define SG_FLAVOUR_SWEEP 16 // class sweep (in-place runs that keep class bytes)
#define SG_FLAVOUR_FORCE 32 // class sweep (and hybrid) on any graph size (see below)
#define SG_FLAVOUR_WPT_SHIFT 6 // bits 6-7: class-sweep warps per tile, 0 = automatic
                              // (sg_sweep_wpt), 1/2/3 = 1/2/4 warps
#define SG_FLAVOUR_HYBRID 256 // class sweep in quiet ticks, the loop form (bits 0-2) in
                              // busy ticks (see SgTickArgs::hybrid_rise/fall and
                              // sg_hybrid_thresholds)
#define SG_FLAVOUR_FLAT 512   // flat draws in place of the loop form (in-place runs): a
                              // warp lays its agents' draws end to end and each lane
                              // takes an equal share; with SWEEP and HYBRID, both forms
                              // run in one launch
#define SG_FLAVOUR_MAX 1023
// The class sweep runs one warp per tile; below this many tiles per SM it
// leaves SMs idle and the loop form (lazy loads) is used instead, unless
// SG_FLAVOUR_FORCE is set.
#define SG_SWEEP_MIN_TILES_PER_SM 2

// Warps per tile of the class sweep: one warp per tile while there are enough
// tiles to give every SM its 4 resident blocks of 8 warps, else 2 or 4 warps
// share a tile so that smaller graphs still fill the SMs.
// Change-count thresholds of the hybrid count step for a launch over ntiles
// tiles (the crossovers measured on a 10^7-agent power-law epidemic: about one
// change per 400 agents while it grows, one per 60 while it declines). The
// unchosen kernel's launch costs about 2.5 us per tick, which smaller graphs
// do not earn back (measured at 10^6 and 2.5 10^6 agents), so the hybrid runs
// from SG_HYBRID_MIN_TILES_PER_SM tiles per SM.
#define SG_HYBRID_MIN_TILES_PER_SM 24
inline void sg_hybrid_thresholds(int64_t ntiles, int sm_count, int32_t flavour, int32_t *rise, int32_t *fall)
{
    const int64_t n = ntiles * SG_TILE;
    const bool on = (flavour & SG_FLAVOUR_HYBRID) && (flavour & SG_FLAVOUR_SWEEP) &&
                    ((flavour & SG_FLAVOUR_FORCE) || ntiles >= (int64_t)sm_count * SG_HYBRID_MIN_TILES_PER_SM);
    *rise = on ? (int32_t)(n / 400 > 0 ? n / 400 : 1) : 0;
    *fall = on ? (int32_t)(n / 60 > 0 ? n / 60 : 1) : 0;
}

inline int32_t sg_sweep_wpt(int64_t ntiles, int sm_count, int32_t flavour)
{
    const int32_t forced = (flavour >> SG_FLAVOUR_WPT_SHIFT) & 3;
    if (forced) return 1 << (forced - 1);
    const int64_t resident = (int64_t)sm_count * 4;
    if (ntiles >= 8 * resident) return 1;
    if (ntiles >= 4 * resident) return 2;
    return 4;
}

// The count scatter hands a changed agent's transpose row longer than
// SG_SEG_ROW entries to its segment list as pieces of SG_SEG_ROW entries, so no
// warp walks a long row alone. A tick changes each agent at most once, and a
// row of L > SG_SEG_ROW entries gives at most 2 L / SG_SEG_ROW pieces, so a
// tick's list holds at most SG_ROWSEG_CAPACITY(nnz) segments.
#define SG_SEG_ROW 64
#define SG_ROWSEG_CAPACITY(nnz) (2 * (size_t)(nnz) / SG_SEG_ROW + 64)

// One warp's share of the scatter: change-list entries [first, first + count),
// count <= 32 (a tile's changes in runs of 32).
struct SgChunk {
    int32_t first, count;
};

// Part [begin, end) of a changed hub's transpose row, with the change's +-1.
struct SgRowSeg {
    int32_t begin, end, delta, pad;
};

struct SgTickArgs {
    const int32_t *off;     // CSR offsets (global agent index)
    const int32_t *idx;     // CSR indices (global agent index)
    void *buf0, *buf1;      // ping-pong state pair (int32 SIR / float32 opinion)
    const SgSeg *segs;
    const SgTile *tiles;
    int32_t ntiles;
    int32_t r;              // tick relative to the run start
    int32_t flavour;        // count-step flavour (SG_FLAVOUR_* bits)
    int32_t thread_row;     // rows up to this length are scanned by one lane, longer
                            // ones by a warp (0 = default 32)
    const SgMega *mega;     // rows longer than mega_row, scanned by whole blocks
    int32_t nmega;
    int32_t mega_blocks;    // the last mega_blocks blocks of the grid take mega rows
    int32_t mega_row;
    // count strategy
    int32_t *cnt;           // infected-neighbour count per agent
    int32_t *changes;       // change list: agent index, ~agent for I->R; tile t
                            // owns changes[tile.begin .. tile.begin + tile_nch[t])
    int2 *change_rows;      // NULL, or beside each change-list entry the changed agent's
                            // transpose row [begin, end) (end = begin when the row goes
                            // through the long-row segments), so the scatter need not load it
    int32_t *tile_nch;      // [ntiles] changes recorded by each tile this tick
    SgChunk *chunks;        // NULL, or the scatter's work list of non-empty chunks
    int32_t *nchunks;       // [ticks] chunk counts, slot r (zero before the run)
    SgRowSeg *rowsegs;      // NULL, or the scatter's list of long-row segments
    int32_t *nrowsegs;      // [ticks] segment counts, slot r (zero before the run)
    const int32_t *toff;    // transpose CSR (in-neighbours)
    const int32_t *tidx;
    uint8_t *cls;           // NULL, or per agent its class (0 S, 1 I, 2 R, 3 other),
                            // kept in step with the state by every count kernel;
                            // tiles then start at multiples of 32
    uint32_t *amask;        // with cls: bit i set whenever cnt[i] may be > 0 (set by
                            // the init and by the scatter's +1, cleared by the sweep
                            // when it reads 0)
    uint8_t *mrebuild;      // NULL, or [ticks + 1] flags: 1 = the activity bits are not
                            // kept for tick r (the scatter of tick r - 1 had too many
                            // changes to set them), so the sweep of tick r rebuilds
                            // them from the counts; zero before the run
    int32_t *tick_changes;  // with mrebuild: [ticks] changes recorded by the sweep at
                            // tick r (zero before the run)
    int32_t *tick_cand;     // NULL, or [ticks] candidates the sweep processed at tick r
                            // (zero before the run)
    int32_t sweep_wpt;      // class sweep: warps per tile (1, 2 or 4; see sg_sweep_wpt)
    size_t cnt_window;      // count strategy: bytes of cnt to keep in L2 as persisting lines
                            // (an access-policy window on the count kernels); 0 = none
    const float2 *bm_radius; // opinion: NULL, or the 2^23-entry Box-Muller radius table (pairs),
    const uint32_t *bm_rq;   // corrections to the step's float32 radius estimates, and
    const float2 *bm_trig;   // the split cosine tables of sg_launch_opinion_tables
    float sigma_hi, sigma_lo; // opinion: the noise sigma as a double-float pair (with the tables)
    const int32_t *nb8;     // opinion, width 8: NULL, or the neighbour table of
                            // sg_launch_opinion_neighbours8 (SG_NB8_AT)
    const void *l2_win;     // opinion: NULL, or an access-policy window (persisting lines)
    size_t l2_win_bytes;    // over l2_win_bytes from l2_win, a fraction l2_win_hit of its
    float l2_win_hit;       // lines kept (the radius table, read at random)
    int32_t hybrid_rise;    // hybrid count step (0 = off): tick r > 1 runs the loop form
    int32_t hybrid_fall;    // when tick r - 1 recorded more than hybrid_rise changes and
                            // no fewer than tick r - 2 (epidemic growing), or more than
                            // hybrid_fall changes; the class sweep otherwise
    // frontier strategy
    int32_t *list[2];       // active agents of tick r in list[r & 1]
    int32_t *list_len;      // [ticks + 1] list lengths, slot r
    int32_t *nch;           // [ticks] change counts, slot r (changes[] reused per tick)
    int32_t *mark;          // per agent: the last list index it was appended to
    const int32_t *aseg;    // per agent: its segment (NULL = segment 0)
    unsigned long long *stats_init;  // build: S, I, R, E_S at the run start
    unsigned long long *stats_delta; // step: [ticks][4] infections, recoveries, degree sum
};

// Launchers return cudaGetLastError() of the launch.
// variant: 1 = SIR-A, 2 = SIR-B (all segments of one launch share it). stats
// selects the instantiation that accumulates S/I/R counts and E_S into
// seg.stats (segments with stats == NULL skip the flush).
cudaError_t sg_launch_sir_pull(const SgTickArgs &a, int variant, bool stats, int grid,
                               cudaStream_t st);
cudaError_t sg_launch_sir_count_init(const SgTickArgs &a, int grid, cudaStream_t st);
// The same counts (and class bytes and activity bits) built by scattering from
// the infected agents over the transpose rows: two kernels. Only for a step whose
// tiles cover every agent of the graph with one segment; the grid takes no mega
// blocks.
cudaError_t sg_launch_sir_count_init_scatter(const SgTickArgs &a, int grid, cudaStream_t st);
// inplace: the state buffer is read and written in place (buf0); only changed
// agents are stored. Valid when the count step is the engine's only step, since
// it reads nothing but the agent's own state and count.
// nlaunched (optional): kernels launched (2 for the hybrid step, else 1).
cudaError_t sg_launch_sir_count_step(const SgTickArgs &a, int variant, bool stats, bool inplace,
                                     int grid, cudaStream_t st, int *nlaunched = nullptr);
cudaError_t sg_launch_sir_count_scatter(const SgTickArgs &a, int grid, cudaStream_t st);
// Frontier strategy (state in buf0, updated in place). list_len[0..ticks] and
// nch[0..ticks-1] must be zero before the build.
cudaError_t sg_launch_frontier_build(const SgTickArgs &a, bool stats, int grid, cudaStream_t st);
cudaError_t sg_launch_frontier_step(const SgTickArgs &a, int variant, bool stats, int grid, cudaStream_t st);
cudaError_t sg_launch_frontier_scatter(const SgTickArgs &a, int grid, cudaStream_t st);
cudaError_t sg_launch_opinion(const SgTickArgs &a, int grid, cudaStream_t st, int width);
// Fills the opinion step's Box-Muller tables: radius[k] = r(k) = sqrt(-2 log(k /
// 2^23 + 1e-10)) for k < 2^23 as a double-float pair (hi, lo) of float32 (64
// MiB), rq[k] = (r(k) - e(k)) * 2^40 rounded to an int32 (stored as uint32; 32
// MiB, SG_BM_RQ_BYTES), where e(k) is the opinion step's own float32 estimate of
// r(k), and trig =
// SG_BM_TRIG_ENTRIES pairs: cos of 2 pi j / 2^12 (j < 4096), then cos and sin of
// 2 pi l / 2^23 (l < 2048), from which the step forms cos(2 pi k / 2^23) by angle
// addition. radius NULL: only the cosine tables are filled; rq NULL: no
// fixed-point radii.
#define SG_BOX_MULLER_SIZE (1 << 23)
#define SG_BM_TRIG_ENTRIES (4096 + 2 * 2048)
#define SG_BM_RQ_BYTES ((size_t)SG_BOX_MULLER_SIZE * 4)
cudaError_t sg_launch_opinion_tables(float2 *radius, uint32_t *rq, float2 *trig, cudaStream_t st);
// nb8[SG_NB8_AT(i, j)] = indices[offsets[i] + j] for j < min(deg(i), 8), else
// -1: the width-8 opinion step's neighbours, group-major. Agents come in groups
// of 32 (agent i in group i / 32), each group's table is 256 entries (1 KiB):
// its agents' first neighbours, then their second neighbours, and so on. A
// warp's loads of the j-th neighbours of 32 consecutive agents are one 128-byte
// line, and the table of 32 consecutive groups is one contiguous 32 KiB range.
// The table holds SG_NB8_ENTRIES(n) entries (whole groups; the entries of
// agents >= n are -1).
#define SG_NB8_AT(i, j) ((((int64_t)(i) >> 5) << 8) + ((int64_t)(j) << 5) + ((i) & 31))
#define SG_NB8_ENTRIES(n) ((((int64_t)(n) + 31) >> 5) << 8)
cudaError_t sg_launch_opinion_neighbours8(const int32_t *offsets, const int32_t *indices, int64_t n, int32_t *nb8,
                                          cudaStream_t st);
// For q < n: out[q] = the opinion step's noise result for opinion x[q] and the
// draw's integers k1[q], k2[q] < 2^23 (a's Box-Muller tables and sigma set),
// exact[q] = the result with the pair-table radius, slow[q] = 1 where the
// fixed-point radius left the float32 rounding open.
cudaError_t sg_launch_opinion_noise_check(const SgTickArgs &a, const float *x, const uint32_t *k1, const uint32_t *k2,
                                          int64_t n, float *out, float *exact, uint8_t *slow, cudaStream_t st);
// out[2 q] = the split-table cosine of k = k0 + q (hi + lo), out[2 q + 1] =
// cos(2 pi k / 2^23) evaluated directly (q < n).
cudaError_t sg_launch_opinion_cos_check(const float2 *trig, int32_t k0, int32_t n, double *out, cudaStream_t st);
// Adds edge_base to off[0..n1) and agent_base to idx[0..nnz) in place (placing a
// scenario's local CSR into a pool).
cudaError_t sg_launch_offset_csr(int32_t *off, int64_t n1, int32_t edge_base, int32_t *idx, int64_t nnz,
                                 int32_t agent_base, cudaStream_t st);
// Checks a local CSR on the device (offsets[0] and offsets[n] checked by the
// caller): *flag (zeroed by the caller) = 1 if the offsets decrease, 2 if an
// index is outside [0, n).
cudaError_t sg_launch_check_csr(const int32_t *off, int64_t n, const int32_t *idx, int64_t nnz, int32_t *flag,
                                cudaStream_t st);
// Copies [begin, end) of `words` 32-bit words from src to dst (write-back of
// agents outside a step's range).
cudaError_t sg_launch_copy_words(const uint32_t *src, uint32_t *dst, int64_t n, cudaStream_t st);
// Transpose of a CSR (n rows, entries < n): counts, exclusive scan, fill.
// tmp needs n+1 int32. Row order of the result is not specified (the count
// strategy only sums over it).
cudaError_t sg_transpose_csr(const int32_t *off, const int32_t *idx, int64_t n, int64_t nnz,
                             int32_t *toff, int32_t *tidx, int32_t *tmp, void *scan_tmp,
                             size_t scan_tmp_bytes, cudaStream_t st);
size_t sg_transpose_scan_bytes(int64_t n);
