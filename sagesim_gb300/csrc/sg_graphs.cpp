// sg_graphs.cpp -- seeded synthetic graphs, locality partition and CSR permute
// (host code).
//
// SAGESim builds its graphs in user code with networkx and partitions them
// with METIS (sagesim/generate_partition.py:24-69, sagesim/partition_utils.py:
// 39-103); neither is usable at 10^7 agents here (networkx is too slow, METIS
// is absent), so the engine ships its own. Everything is integer arithmetic
// or IEEE basic operations on a splitmix64/xoshiro256** stream, so the same
// seed gives the same graph on x86-64 and aarch64.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include "../../include/sagesim_gb300.h"

namespace {

struct Rng { // xoshiro256** seeded by splitmix64
    uint64_t s[4];
    explicit Rng(uint64_t seed)
    {
        uint64_t z = seed;
        for (auto &w : s) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            w = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next()
    {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform in [0, n) without modulo bias (Lemire's method)
    uint64_t below(uint64_t n)
    {
        if (n <= 1) return 0;
        const uint64_t thresh = (0 - n) % n;
        for (;;) {
            const uint64_t x = next();
            const __uint128_t m = (__uint128_t)x * n;
            if ((uint64_t)m >= thresh) return (uint64_t)(m >> 64);
        }
    }
    // uniform double in [0, 1) with 53 random bits
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Natural log from IEEE basic operations only (no libm), so geometric skips
// are identical across platforms: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(t), t = (m-1)/(m+1), series to t^41 (|t| < 0.172).
double det_log(double x)
{
    int e = 0;
    while (x >= 1.4142135623730951) {
        x *= 0.5;
        ++e;
    }
    while (x < 0.7071067811865476) {
        x *= 2.0;
        --e;
    }
    const double t = (x - 1.0) / (x + 1.0);
    const double t2 = t * t;
    double term = t, sum = 0.0;
    for (int k = 1; k <= 41; k += 2) {
        sum += term / (double)k;
        term *= t2;
    }
    return 2.0 * sum + (double)e * 0.6931471805599453;
}

struct EdgeList {
    std::vector<int32_t> a, b;
    void add(int32_t x, int32_t y)
    {
        a.push_back(x);
        b.push_back(y);
    }
};

// Symmetric CSR from an undirected edge list; row order = edge insertion
// order (each edge (x, y) appends y to row x and x to row y), duplicates and
// self loops dropped (first occurrence kept).
int to_csr(int64_t n, const EdgeList &el, int32_t *offsets, int32_t *indices, int64_t *nnz,
           bool dedup)
{
    const size_t m = el.a.size();
    std::vector<int64_t> deg(n + 1, 0);
    for (size_t k = 0; k < m; ++k) {
        if (el.a[k] == el.b[k]) continue;
        deg[el.a[k]]++;
        deg[el.b[k]]++;
    }
    std::vector<int64_t> off(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) off[i + 1] = off[i] + deg[i];
    std::vector<int32_t> idx(off[n]);
    std::vector<int64_t> cur(off.begin(), off.end() - 1);
    for (size_t k = 0; k < m; ++k) {
        const int32_t x = el.a[k], y = el.b[k];
        if (x == y) continue;
        idx[cur[x]++] = y;
        idx[cur[y]++] = x;
    }
    // drop duplicates in place, keeping first occurrences in row order
    int64_t total = 0;
    std::vector<int64_t> noff(n + 1, 0);
    if (dedup) {
        std::vector<int32_t> mark(n, -1);
        int64_t w = 0;
        for (int64_t i = 0; i < n; ++i) {
            noff[i] = w;
            for (int64_t k = off[i]; k < off[i + 1]; ++k) {
                const int32_t j = idx[k];
                if (mark[j] == (int32_t)i) continue;
                mark[j] = (int32_t)i;
                idx[w++] = j;
            }
        }
        noff[n] = w;
        total = w;
    } else {
        noff = off;
        total = off[n];
    }
    if (total >= INT32_MAX) return SG_ERR_INVALID;
    *nnz = total;
    if (offsets) {
        for (int64_t i = 0; i <= n; ++i) offsets[i] = (int32_t)noff[i];
    }
    if (indices && total) memcpy(indices, idx.data(), (size_t)total * sizeof(int32_t));
    return SG_OK;
}

} // namespace

extern "C" {

// G(n, p): pairs (i < j) in lexicographic order, gaps between edges drawn
// geometrically: skip = floor(log(U) / log(1 - p)).
int sg_graph_er(int64_t n, double p, uint64_t seed, int32_t *offsets, int32_t *indices, int64_t *nnz)
{
    if (n < 0 || n >= INT32_MAX || !(p >= 0.0 && p <= 1.0) || !nnz) return SG_ERR_INVALID;
    Rng rng(seed);
    EdgeList el;
    if (p > 0.0 && n > 1) {
        const double lq = det_log(1.0 - p);
        int64_t v = 1, w = -1;
        while (v < n) {
            double u = rng.unit();
            if (u <= 0.0) u = 1e-300;
            const double skip = p >= 1.0 ? 0.0 : det_log(u) / lq;
            w += 1 + (int64_t)skip;
            while (w >= v && v < n) {
                w -= v;
                ++v;
            }
            if (v < n) el.add((int32_t)v, (int32_t)w);
        }
    }
    return to_csr(n, el, offsets, indices, nnz, true);
}

// Barabasi-Albert: nodes 0..m-1 start without edges; node m connects to all
// of them; every later node t attaches to m distinct targets drawn with
// probability proportional to degree (uniform picks from the list of edge
// endpoints, repeats rejected).
int sg_graph_ba(int64_t n, int32_t m, uint64_t seed, int32_t *offsets, int32_t *indices, int64_t *nnz)
{
    if (n < 0 || n >= INT32_MAX || m < 1 || !nnz) return SG_ERR_INVALID;
    if (n <= m) return to_csr(n, EdgeList{}, offsets, indices, nnz, true);
    Rng rng(seed);
    EdgeList el;
    el.a.reserve((size_t)(n - m) * m);
    el.b.reserve((size_t)(n - m) * m);
    std::vector<int32_t> ends;
    ends.reserve((size_t)(n - m) * m * 2);
    std::vector<int32_t> targets(m);
    for (int32_t k = 0; k < m; ++k) targets[k] = k;
    std::vector<int64_t> stamp(n, -1);
    for (int64_t t = m; t < n; ++t) {
        for (int32_t k = 0; k < m; ++k) {
            el.add((int32_t)t, targets[k]);
            ends.push_back((int32_t)t);
            ends.push_back(targets[k]);
        }
        // next node's m distinct targets
        if (t + 1 < n) {
            int32_t got = 0;
            while (got < m) {
                const int32_t c = ends[rng.below(ends.size())];
                if (stamp[c] == t) continue;
                stamp[c] = t;
                targets[got++] = c;
            }
        }
    }
    return to_csr(n, el, offsets, indices, nnz, true);
}

// Watts-Strogatz: ring lattice, each node joined to k/2 successors; each
// lattice edge (u, u+j) is then, with probability p, rewired to (u, w) for a
// uniform w that is neither u nor already a neighbour of u (tries up to n
// times, then keeps the edge). Rows list neighbours in insertion order.
int sg_graph_ws(int64_t n, int32_t k, double p, uint64_t seed, int32_t *offsets, int32_t *indices,
                int64_t *nnz)
{
    if (n < 0 || n >= INT32_MAX || k < 0 || (k & 1) || !(p >= 0.0 && p <= 1.0) || !nnz)
        return SG_ERR_INVALID;
    if (k >= n) k = (int32_t)((n - 1) & ~1LL);
    if (k < 0) k = 0;
    Rng rng(seed);
    const int32_t half = k / 2;
    // adjacency as sorted small vectors for duplicate checks
    std::vector<std::vector<int32_t>> adj(n);
    auto has = [&](int64_t u, int32_t v) {
        const auto &a = adj[u];
        return std::find(a.begin(), a.end(), v) != a.end();
    };
    std::vector<int32_t> ea, eb;
    ea.reserve((size_t)n * half);
    eb.reserve((size_t)n * half);
    for (int64_t u = 0; u < n; ++u)
        for (int32_t j = 1; j <= half; ++j) {
            const int32_t v = (int32_t)((u + j) % n);
            ea.push_back((int32_t)u);
            eb.push_back(v);
            adj[u].push_back(v);
            adj[v].push_back((int32_t)u);
        }
    const uint64_t pthresh = p >= 1.0 ? UINT64_MAX : (uint64_t)(p * 18446744073709551616.0);
    for (size_t q = 0; q < ea.size(); ++q) {
        const bool rewire = p >= 1.0 || rng.next() < pthresh;
        if (!rewire) continue;
        const int32_t u = ea[q], v = eb[q];
        int32_t w = -1;
        for (int64_t tries = 0; tries < n; ++tries) {
            const int32_t c = (int32_t)rng.below((uint64_t)n);
            if (c != u && !has(u, c)) {
                w = c;
                break;
            }
        }
        if (w < 0) continue;
        auto &au = adj[u];
        au.erase(std::find(au.begin(), au.end(), v));
        auto &av = adj[v];
        av.erase(std::find(av.begin(), av.end(), u));
        au.push_back(w);
        adj[w].push_back(u);
        eb[q] = w;
    }
    EdgeList el;
    el.a.swap(ea);
    el.b.swap(eb);
    return to_csr(n, el, offsets, indices, nnz, true);
}

// Seeded k-way graph-growing partition used as a locality relabelling.
// k seeds are drawn uniformly; parts grow by BFS in round-robin, each part
// capped at ceil(n/k) agents; agents left unreached (other components) start
// new BFS waves into the least-filled part. New indices are assigned part by
// part, in BFS discovery order inside a part, so neighbours tend to get nearby
// indices (what a METIS-ordered relabel gives the neighbour gathers).
int sg_partition_relabel(int64_t n, const int32_t *offsets, const int32_t *indices, int32_t k,
                         uint64_t seed, int32_t *perm, int32_t *part)
{
    if (n < 0 || n >= INT32_MAX || k < 1 || !offsets || !perm) return SG_ERR_INVALID;
    if (n == 0) return SG_OK;
    if (k > n) k = (int32_t)n;
    Rng rng(seed);
    const int64_t cap = (n + k - 1) / k;
    std::vector<int32_t> owner(n, -1);
    std::vector<int64_t> size(k, 0);
    std::vector<std::vector<int32_t>> order(k);
    std::vector<std::queue<int32_t>> frontier(k);
    for (int32_t p = 0; p < k; ++p) {
        for (int tries = 0; tries < 64; ++tries) {
            const int32_t s = (int32_t)rng.below((uint64_t)n);
            if (owner[s] < 0) {
                owner[s] = p;
                size[p] = 1;
                order[p].push_back(s);
                frontier[p].push(s);
                break;
            }
        }
    }
    int64_t assigned = 0;
    for (int32_t p = 0; p < k; ++p) assigned += size[p];
    int64_t scan = 0;
    while (assigned < n) {
        bool progressed = false;
        for (int32_t p = 0; p < k; ++p) {
            // expand one frontier node per round per part
            while (!frontier[p].empty() && size[p] < cap) {
                const int32_t u = frontier[p].front();
                frontier[p].pop();
                bool any = false;
                for (int32_t q = offsets[u]; q < offsets[u + 1] && size[p] < cap; ++q) {
                    const int32_t v = indices[q];
                    if (owner[v] >= 0) continue;
                    owner[v] = p;
                    size[p]++;
                    order[p].push_back(v);
                    frontier[p].push(v);
                    ++assigned;
                    any = true;
                }
                if (any) {
                    progressed = true;
                    break;
                }
            }
        }
        if (!progressed) {
            // restart from the next unassigned agent in the least-filled part
            while (scan < n && owner[scan] >= 0) ++scan;
            if (scan >= n) break;
            int32_t best = 0;
            for (int32_t p = 1; p < k; ++p)
                if (size[p] < size[best]) best = p;
            if (size[best] >= cap) {
                // all parts full (rounding): put the rest into the last part
                best = k - 1;
            }
            owner[scan] = best;
            size[best]++;
            order[best].push_back((int32_t)scan);
            while (!frontier[best].empty()) frontier[best].pop();
            frontier[best].push((int32_t)scan);
            ++assigned;
        }
    }
    int32_t next = 0;
    for (int32_t p = 0; p < k; ++p)
        for (int32_t v : order[p]) {
            perm[v] = next;
            if (part) part[next] = p;
            ++next;
        }
    return next == (int32_t)n ? SG_OK : SG_ERR_INVALID;
}

int sg_csr_permute(int64_t n, const int32_t *offsets, const int32_t *indices, const int32_t *perm,
                   int32_t *new_offsets, int32_t *new_indices)
{
    if (n < 0 || !offsets || !perm || !new_offsets) return SG_ERR_INVALID;
    std::vector<int32_t> inv(n);
    std::vector<char> seen(n, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int32_t p = perm[i];
        if (p < 0 || p >= n || seen[p]) return SG_ERR_INVALID;
        seen[p] = 1;
        inv[p] = (int32_t)i;
    }
    new_offsets[0] = 0;
    for (int64_t j = 0; j < n; ++j) {
        const int32_t i = inv[j];
        new_offsets[j + 1] = new_offsets[j] + (offsets[i + 1] - offsets[i]);
    }
    if (new_indices) {
        for (int64_t j = 0; j < n; ++j) {
            const int32_t i = inv[j];
            int32_t w = new_offsets[j];
            for (int32_t q = offsets[i]; q < offsets[i + 1]; ++q) new_indices[w++] = perm[indices[q]];
        }
    }
    return SG_OK;
}

} // extern "C"
