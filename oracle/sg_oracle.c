/*
 * sg_oracle.c -- CPU restatement of SAGESim's per-tick agent step.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker the CUDA engine is
 * compared against; nothing in the product links or calls it. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Parity pins: the Philox restatement is checked against vectors produced by
 * the reference's own rand_uniform_philox / rand_normal run through a CPU
 * stand-in for cupyx.jit (tests/golden/philox_vectors.json), and the tick
 * semantics against per-tick agent states produced by the reference's own
 * Model.setup()/simulate() pipeline on the same inputs (the .npz fixtures in tests/golden).
 *
 * Compile with -ffp-contract=off: the opinion step's float32 arithmetic must
 * round after every multiply and add, as the reference's typed operations do.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Philox-2x32-10 with SAGESim's counter layout.
 * sagesim/math_utils.py:106-189 (rand_uniform_philox):
 *   c0 = (tick*1000003 + salt) mod 2^32, c1 = agent mod 2^32, key = seed mod 2^32;
 *   ten rounds of (c0,c1) <- (hi(M*c0) ^ key ^ c1, lo(M*c0)),
 *   key += 0x9E3779B9 after rounds 1..9; result = (c0 mod 2^23) / 2^23.
 * M is the literal the reference multiplies by, 3529668003 = 0xD26275A3
 * (math_utils.py:111 and each later round). Its header comment
 * (math_utils.py:81) names 0xD256D193, the Random123 constant, but the code
 * uses 0xD26275A3, so that is the value that defines the reference's stream.
 * The reference computes in Python/CuPy int64 with floor-div/mod; the int64 wrap
 * of M*c0 does not change hi/lo mod 2^32, so uint32 arithmetic gives the same
 * bits. Returns the 23-bit integer k; the uniform is k / 2^23 exactly. */
uint32_t sgo_philox_k23(int64_t seed, int64_t tick, int64_t lid, int64_t salt)
{
    uint32_t c0 = (uint32_t)(uint64_t)(tick * 1000003LL + salt);
    uint32_t c1 = (uint32_t)(uint64_t)lid;
    uint32_t key = (uint32_t)(uint64_t)seed;
    for (int r = 0; r < 10; ++r) {
        uint64_t p = (uint64_t)c0 * 0xD26275A3ULL;
        uint32_t hi = (uint32_t)(p >> 32);
        uint32_t lo = (uint32_t)p;
        c0 = hi ^ key ^ c1;
        c1 = lo;
        if (r < 9) key += 0x9E3779B9U;
    }
    return c0 & 0x7FFFFFU;
}

double sgo_rand_uniform(int64_t seed, int64_t tick, int64_t lid, int64_t salt)
{
    return (double)sgo_philox_k23(seed, tick, lid, salt) / 8388608.0;
}

/* sagesim/math_utils.py:231-255 (rand_normal): Box-Muller in double,
 * u1 with salt, u2 with salt + 73856093, log guarded by +1e-10. */
double sgo_rand_normal(int64_t seed, int64_t tick, int64_t lid, int64_t salt)
{
    double u1 = sgo_rand_uniform(seed, tick, lid, salt);
    double u2 = sgo_rand_uniform(seed, tick, lid, salt + 73856093LL);
    double u1s = u1 + 1e-10;
    return sqrt(-2.0 * log(u1s)) * cos(6.283185307179586 * u2);
}

/* Integer threshold for `u < p` with u = k/2^23 and p a float64 global
 * (sagesim/model.py:593 stores globals as float64). k/2^23 < p  <=>  k < p*2^23
 * (scaling by 2^23 is exact)  <=>  k < ceil(p*2^23). NaN or p <= 0 -> 0. */
uint32_t sgo_threshold(double p)
{
    double x = ldexp(p, 23);
    if (!(x > 0.0)) return 0u;
    if (x >= 8388608.0) return 8388608u;
    return (uint32_t)ceil(x);
}

/* One SIR tick for every agent in [0, n).
 *
 * variant 1 (reference test step, tests/test_simulation.py:24-43):
 *   u = philox(seed, tick, lid, 1); I and u<gamma -> R; S: if any neighbour is I
 *   and u<beta -> I. (The reference scans every neighbour; the outcome depends
 *   only on "any I neighbour".)
 * variant 2 (per-infected-neighbour trials, the step in
 *   tests/golden/ref_steps.py run through the reference pipeline):
 *   I: u = philox(salt 1), u<gamma -> R. S: scanning neighbours in CSR order, the
 *   j-th infected neighbour found (j = 0, 1, ...) draws philox(salt 2+j); the
 *   first draw below beta infects and stops the scan.
 * Reads see tick-start states (sin); writes go to sout -- the reference's double
 * buffer (sagesim/model.py:2142-2220 write_* redirection, write-back at
 * model.py:2374-2408). Agents with any other state value are copied unchanged.
 *
 * stats (nullable): [S, I, R] counts after the tick and E_S = sum of degrees of
 * agents susceptible at tick start (the reference's neighbour-scan set).
 * lids (nullable): RNG key per agent; NULL means the agent index
 * (sagesim/model.py:1089-1096 defaults logical ids to agent ids). */
void sgo_sir_tick(int variant, int64_t n, const int32_t *off, const int32_t *idx,
                  const int64_t *lids, int64_t seed, int64_t tick, double beta,
                  double gamma, int32_t cs, int32_t ci, int32_t cr,
                  const int32_t *sin, int32_t *sout, int64_t *stats)
{
    const uint32_t kinf = sgo_threshold(beta);
    const uint32_t krec = sgo_threshold(gamma);
    int64_t nS = 0, nI = 0, nR = 0, eS = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : nS, nI, nR, eS)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t s = sin[i];
        const int64_t lid = lids ? lids[i] : i;
        int32_t out = s;
        if (s == ci) {
            if (sgo_philox_k23(seed, tick, lid, 1) < krec) out = cr;
        } else if (s == cs) {
            const int32_t b = off[i], e = off[i + 1];
            eS += (int64_t)(e - b);
            if (variant == 1) {
                if (sgo_philox_k23(seed, tick, lid, 1) < kinf) {
                    for (int32_t k = b; k < e; ++k) {
                        if (sin[idx[k]] == ci) { out = ci; break; }
                    }
                }
            } else {
                int64_t j = 0;
                for (int32_t k = b; k < e; ++k) {
                    if (sin[idx[k]] == ci) {
                        if (sgo_philox_k23(seed, tick, lid, 2 + j) < kinf) { out = ci; break; }
                        ++j;
                    }
                }
            }
        }
        sout[i] = out;
        nS += (out == cs);
        nI += (out == ci);
        nR += (out == cr);
    }
    if (stats) { stats[0] = nS; stats[1] = nI; stats[2] = nR; stats[3] = eS; }
}

/* Runs nticks ticks starting at tick0; state is updated in place. stats
 * (nullable) receives 4 int64 per tick; history (nullable) receives the state
 * after each tick as int8 (n per tick). Returns 0, or -1 on allocation failure. */
int sgo_sir_run(int variant, int64_t n, const int32_t *off, const int32_t *idx,
                const int64_t *lids, int64_t seed, int64_t tick0, int32_t nticks,
                double beta, double gamma, int32_t cs, int32_t ci, int32_t cr,
                int32_t *state, int64_t *stats, int8_t *history, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int32_t *tmp = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    if (!tmp) return -1;
    for (int32_t t = 0; t < nticks; ++t) {
        sgo_sir_tick(variant, n, off, idx, lids, seed, tick0 + t, beta, gamma, cs, ci, cr,
                     state, tmp, stats ? stats + 4 * (int64_t)t : NULL);
        memcpy(state, tmp, (size_t)n * sizeof(int32_t));
        if (history) {
            int8_t *h = history + (int64_t)t * n;
            for (int64_t i = 0; i < n; ++i) h[i] = (int8_t)state[i];
        }
    }
    free(tmp);
    return 0;
}

/* Opinion step (float32 property + padded float32[8] list property, ordered
 * neighbours). The step is the one in tests/golden/ref_steps.py run through the
 * reference pipeline:
 *   m = min(deg, width); acc = sum_{j<m} w[i][j] * x[nbr_j]  (float32, in order)
 *   norm = sum_{j<m} |w[i][j]|  (float32, in order)
 *   x' = norm > 0 ? acc / norm : x[i]                         (float32)
 *   y = (double)x' + sigma * rand_normal(seed, tick, lid, 1)  (float64)
 *   y clamped to [0, 1] in double, stored as float32.
 * Every float32 multiply and add rounds separately (no fused multiply-add). */
void sgo_opinion_tick(int64_t n, const int32_t *off, const int32_t *idx, const int64_t *lids,
                      int64_t seed, int64_t tick, double sigma, int32_t width,
                      const float *w, const float *xin, float *xout)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t b = off[i];
        int32_t m = off[i + 1] - b;
        if (m > width) m = width;
        float acc = 0.0f, norm = 0.0f;
        for (int32_t j = 0; j < m; ++j) {
            const float wj = w[i * (int64_t)width + j];
            const float prod = wj * xin[idx[b + j]];
            acc = acc + prod;
            norm = norm + fabsf(wj);
        }
        float x = xin[i];
        if (norm > 0.0f) x = acc / norm;
        const int64_t lid = lids ? lids[i] : i;
        double y = (double)x + sigma * sgo_rand_normal(seed, tick, lid, 1);
        if (y < 0.0) y = 0.0;
        if (y > 1.0) y = 1.0;
        xout[i] = (float)y;
    }
}

int sgo_opinion_run(int64_t n, const int32_t *off, const int32_t *idx, const int64_t *lids,
                    int64_t seed, int64_t tick0, int32_t nticks, double sigma, int32_t width,
                    const float *w, float *x, float *history, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    float *tmp = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    if (!tmp) return -1;
    for (int32_t t = 0; t < nticks; ++t) {
        sgo_opinion_tick(n, off, idx, lids, seed, tick0 + t, sigma, width, w, x, tmp);
        memcpy(x, tmp, (size_t)n * sizeof(float));
        if (history) memcpy(history + (int64_t)t * n, x, (size_t)n * sizeof(float));
    }
    free(tmp);
    return 0;
}

/* ---- input generator for the CPU baseline -------------------------------
 * The reference builds its graphs in user code (networkx, e.g.
 * scaling_tests/weak_scaling_sir.py builds its SIR graphs before timing
 * simulate()); networkx takes minutes and tens of GB at 10^7 agents, so the
 * benchmark's Barabasi-Albert input is written out here from its published
 * definition, so that the CPU baseline builds its input without the engine's
 * library. The stream is xoshiro256** seeded through splitmix64 (Blackman &
 * Vigna), bounded draws by Lemire's multiply-shift rejection method; the
 * attachment rule is the usual linear preferential attachment: node m joins
 * nodes 0..m-1, every later node t joins m distinct nodes drawn uniformly
 * from the list of all edge endpoints so far (repeats redrawn). Rows list
 * neighbours in edge order. The engine's generator follows the same
 * definition; a CPU test checks that both give the same CSR. */
typedef struct { uint64_t s[4]; } sgo_xoshiro;

static void sgo_xoshiro_seed(sgo_xoshiro *r, uint64_t seed)
{
    uint64_t z = seed;
    for (int k = 0; k < 4; ++k) {
        z += 0x9E3779B97F4A7C15ULL;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
        r->s[k] = x ^ (x >> 31);
    }
}

static inline uint64_t sgo_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t sgo_xoshiro_next(sgo_xoshiro *r)
{
    uint64_t *s = r->s;
    const uint64_t out = sgo_rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = sgo_rotl(s[3], 45);
    return out;
}

static uint64_t sgo_below(sgo_xoshiro *r, uint64_t bound)
{
    if (bound <= 1) return 0;
    const uint64_t reject_below = (0 - bound) % bound;
    for (;;) {
        const unsigned __int128 m = (unsigned __int128)sgo_xoshiro_next(r) * bound;
        if ((uint64_t)m >= reject_below) return (uint64_t)(m >> 64);
    }
}

/* Barabasi-Albert graph as a symmetric CSR. Call with offsets == NULL to get
 * nnz only, then again with offsets[n+1] and indices[nnz]. Returns 0, -1 on a
 * bad argument, -2 when out of memory. */
int sgo_graph_ba(int64_t n, int32_t m, uint64_t seed, int32_t *offsets, int32_t *indices, int64_t *nnz)
{
    if (n < 0 || n >= INT32_MAX || m < 1 || !nnz) return -1;
    if (n <= m) {
        *nnz = 0;
        if (offsets) memset(offsets, 0, (size_t)(n + 1) * sizeof(int32_t));
        return 0;
    }
    const int64_t nedges = (n - m) * (int64_t)m;
    if (2 * nedges >= INT32_MAX) return -1;
    *nnz = 2 * nedges;
    if (!offsets) return 0;
    /* edge k joins src[k] = m + k / m to dst[k]; endpoints list for the draws */
    int32_t *dst = (int32_t *)malloc((size_t)nedges * sizeof(int32_t));
    int32_t *ends = (int32_t *)malloc((size_t)(2 * nedges) * sizeof(int32_t));
    int64_t *stamp = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int32_t *tgt = (int32_t *)malloc((size_t)m * sizeof(int32_t));
    if (!dst || !ends || !stamp || !tgt) {
        free(dst); free(ends); free(stamp); free(tgt);
        return -2;
    }
    for (int64_t i = 0; i < n; ++i) stamp[i] = -1;
    for (int32_t k = 0; k < m; ++k) tgt[k] = k;
    sgo_xoshiro rng;
    sgo_xoshiro_seed(&rng, seed);
    int64_t ne = 0, nend = 0;
    for (int64_t t = m; t < n; ++t) {
        for (int32_t k = 0; k < m; ++k) {
            dst[ne++] = tgt[k];
            ends[nend++] = (int32_t)t;
            ends[nend++] = tgt[k];
        }
        if (t + 1 < n) {
            int32_t got = 0;
            while (got < m) {
                const int32_t c = ends[sgo_below(&rng, (uint64_t)nend)];
                if (stamp[c] == t) continue;
                stamp[c] = t;
                tgt[got++] = c;
            }
        }
    }
    free(ends);
    free(stamp);
    free(tgt);
    /* rows in edge order: edge (t, d) appends d to row t and t to row d; the
     * m targets of a node are distinct, so no pair repeats */
    memset(offsets, 0, (size_t)(n + 1) * sizeof(int32_t));
    for (int64_t k = 0; k < nedges; ++k) {
        offsets[m + k / m + 1]++;
        offsets[dst[k] + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) offsets[i + 1] += offsets[i];
    if (indices) {
        int32_t *cur = (int32_t *)malloc((size_t)n * sizeof(int32_t));
        if (!cur) {
            free(dst);
            return -2;
        }
        memcpy(cur, offsets, (size_t)n * sizeof(int32_t));
        for (int64_t k = 0; k < nedges; ++k) {
            const int32_t s = (int32_t)(m + k / m), d = dst[k];
            indices[cur[s]++] = d;
            indices[cur[d]++] = s;
        }
        free(cur);
    }
    free(dst);
    return 0;
}

/* Bulk RNG helpers for vector checks. */
void sgo_philox_batch(int64_t count, const int64_t *seed, const int64_t *tick,
                      const int64_t *lid, const int64_t *salt, uint32_t *k23_out)
{
    for (int64_t i = 0; i < count; ++i) k23_out[i] = sgo_philox_k23(seed[i], tick[i], lid[i], salt[i]);
}

void sgo_normal_batch(int64_t count, const int64_t *seed, const int64_t *tick,
                      const int64_t *lid, const int64_t *salt, double *out)
{
    for (int64_t i = 0; i < count; ++i) out[i] = sgo_rand_normal(seed[i], tick[i], lid[i], salt[i]);
}

int sgo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
