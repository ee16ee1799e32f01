// sg_setup.cu -- graph setup on the GPU: agent ids -> buffer indices through an
// open-addressing hash table in HBM, and the CSR built by sorting the mapped edges.
//
// Replaces the reference's host-side id conversion (convert_agent_ids_to_indices,
// sagesim/model.py:31-110, which builds a GPU hash map it then reads on the host)
// and its CSR build from per-agent neighbour lists (sagesim/internal_utils.py:111-186).
// Steps, all on the device:
//   1. insert: ids[i] -> i into a table of 2^k >= 2n slots (64-bit keys, linear
//      probing, atomicCAS on the key; a repeated id is an error);
//   2. map: every edge's endpoints looked up (an unknown id is an error) and packed
//      as (src << 32 | dst), plus (dst << 32 | src) for undirected graphs, in call
//      order;
//   3. rows: unordered graphs sort the packed keys and drop repeats (rows sorted by
//      neighbour index, like a neighbour set); ordered graphs sort (src, dst) with the
//      edge position as value, keep each pair's first position, and sort again by
//      (src, position), so a row lists neighbours in first-connection order without
//      repeats (NetworkSpace(ordered=True));
//   4. offsets: per-row counts and an exclusive scan.
// Every probe loop is bounded by the table size.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <string>

#include "sg_internal.h"
#include "sg_setup.h"

namespace {

constexpr unsigned long long kEmptyKey = 0x8000000000000000ull; // INT64_MIN marks an empty slot

// splitmix64's output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", 2014) as the slot hash
__device__ __forceinline__ unsigned long long slot_hash(unsigned long long x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__global__ void id_insert_kernel(const long long *__restrict__ ids, long long n, unsigned long long *keys,
                                 int32_t *vals, unsigned long long mask, int32_t *err)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long key = (unsigned long long)ids[i];
        unsigned long long h = slot_hash(key) & mask;
        for (unsigned long long probe = 0; probe <= mask; ++probe) {
            const unsigned long long prev = atomicCAS(keys + h, kEmptyKey, key);
            if (prev == kEmptyKey) {
                vals[h] = (int32_t)i;
                break;
            }
            if (prev == key) {
                atomicExch(err, 1); // repeated id
                break;
            }
            h = (h + 1) & mask;
        }
    }
}

__device__ __forceinline__ int32_t id_find(const unsigned long long *keys, const int32_t *vals,
                                           unsigned long long mask, unsigned long long key)
{
    unsigned long long h = slot_hash(key) & mask;
    for (unsigned long long probe = 0; probe <= mask; ++probe) {
        const unsigned long long k = keys[h];
        if (k == key) return vals[h];
        if (k == kEmptyKey) return -1;
        h = (h + 1) & mask;
    }
    return -1;
}

// Packs mapped edges. Undirected: edge e writes slots 2e (forward) and 2e + 1
// (reverse), so call order survives a stable sort by source.
__global__ void edge_map_kernel(const long long *__restrict__ src, const long long *__restrict__ dst, long long m,
                                const unsigned long long *keys, const int32_t *vals, unsigned long long mask,
                                bool undirected, unsigned long long *packed, int32_t *err)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
        const int32_t s = id_find(keys, vals, mask, (unsigned long long)src[e]);
        const int32_t d = id_find(keys, vals, mask, (unsigned long long)dst[e]);
        if (s < 0 || d < 0) {
            atomicExch(err, 2); // unknown id
            continue;
        }
        const unsigned long long fwd = ((unsigned long long)(uint32_t)s << 32) | (uint32_t)d;
        if (undirected) {
            packed[2 * e] = fwd;
            packed[2 * e + 1] = ((unsigned long long)(uint32_t)d << 32) | (uint32_t)s;
        } else {
            packed[e] = fwd;
        }
    }
}

__global__ void fill_kernel(unsigned long long *v, long long m, unsigned long long x)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
        v[i] = x;
}

__global__ void iota_kernel(uint32_t *v, long long m)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
        v[i] = (uint32_t)i;
}

// keep[i] = 1 where sorted key i differs from key i - 1 (first of a run)
__global__ void first_of_run_kernel(const unsigned long long *k, long long m, int32_t *keep)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
        keep[i] = (i == 0 || k[i] != k[i - 1]) ? 1 : 0;
}

// Compacts the kept entries: out position = exclusive scan of keep. For ordered
// rows the kept (src, dst) pairs are re-keyed as (src << 32 | first position).
__global__ void compact_kernel(const unsigned long long *k, const uint32_t *pos, const int32_t *keep,
                               const int32_t *at, long long m, bool ordered, unsigned long long *out_key,
                               uint32_t *out_dst)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        const int32_t o = at[i];
        if (ordered) {
            out_key[o] = (k[i] & 0xFFFFFFFF00000000ull) | pos[i];
            out_dst[o] = (uint32_t)(k[i] & 0xFFFFFFFFull);
        } else {
            out_key[o] = k[i];
        }
    }
}

__global__ void row_count_kernel(const unsigned long long *k, long long m, int32_t *cnt)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + (int32_t)(k[i] >> 32), 1);
}

__global__ void low_word_kernel(const unsigned long long *k, long long m, int32_t *idx)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x)
        idx[i] = (int32_t)(k[i] & 0xFFFFFFFFull);
}

// Blocks of 256 threads for `work` items, at most 16 per SM of the current
// device (grid-stride loops).
int grid_of(long long work)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        sms = 1; // the launch that follows reports the device's error
    const long long b = (work + 255) / 256;
    return (int)std::max<long long>(1, std::min<long long>(b, (long long)sms * 16));
}

struct Buf {
    void *p = nullptr;
    ~Buf()
    {
        if (p) cudaFree(p);
    }
    cudaError_t get(size_t bytes)
    {
        return cudaMalloc(&p, std::max<size_t>(bytes, 16));
    }
    template <typename T> T *as() const { return (T *)p; }
};

} // namespace

#define SU_CK(x)                                                                                   \
    do {                                                                                           \
        cudaError_t _e = (x);                                                                      \
        if (_e != cudaSuccess) {                                                                   \
            *why = std::string(#x) + ": " + cudaGetErrorString(_e);                                \
            return SG_ERR_CUDA;                                                                    \
        }                                                                                          \
    } while (0)

int sg_build_csr_from_ids(const int64_t *ids, int64_t n, const int64_t *src, const int64_t *dst, int64_t m,
                          bool undirected, bool ordered, cudaStream_t st, int32_t **d_off, int32_t **d_idx,
                          int64_t *nnz_out, std::string *why)
{
    *d_off = *d_idx = nullptr;
    *nnz_out = 0;
    if (n < 0 || m < 0) {
        *why = "negative agent or edge count";
        return SG_ERR_INVALID;
    }
    const long long mm = undirected ? 2 * (long long)m : (long long)m;
    if (n >= (1LL << 31) - 1 || mm >= (1LL << 32) - 1) {
        *why = "too many agents or edges for 32-bit indices";
        return SG_ERR_INVALID;
    }
    for (int64_t i = 0; i < n; ++i)
        if ((unsigned long long)ids[i] == kEmptyKey) {
            *why = "agent id INT64_MIN is reserved";
            return SG_ERR_INVALID;
        }
    unsigned long long cap = 1;
    while (cap < 2ull * (unsigned long long)std::max<int64_t>(n, 1)) cap <<= 1;
    Buf dids, dsrc, ddst, keys, vals, err, packed, pos, keep, at, key2, dst2, sortk, sortv, cnt, tmp;
    SU_CK(dids.get((size_t)n * 8));
    SU_CK(dsrc.get((size_t)m * 8));
    SU_CK(ddst.get((size_t)m * 8));
    SU_CK(keys.get((size_t)cap * 8));
    SU_CK(vals.get((size_t)cap * 4));
    SU_CK(err.get(4));
    if (n) SU_CK(cudaMemcpyAsync(dids.p, ids, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    if (m) SU_CK(cudaMemcpyAsync(dsrc.p, src, (size_t)m * 8, cudaMemcpyHostToDevice, st));
    if (m) SU_CK(cudaMemcpyAsync(ddst.p, dst, (size_t)m * 8, cudaMemcpyHostToDevice, st));
    SU_CK(cudaMemsetAsync(err.p, 0, 4, st));
    fill_kernel<<<grid_of((long long)cap), 256, 0, st>>>(keys.as<unsigned long long>(), (long long)cap, kEmptyKey);
    SU_CK(cudaGetLastError());
    if (n) id_insert_kernel<<<grid_of(n), 256, 0, st>>>(dids.as<long long>(), n, keys.as<unsigned long long>(),
                                                         vals.as<int32_t>(), cap - 1, err.as<int32_t>());
    SU_CK(cudaGetLastError());
    SU_CK(packed.get((size_t)mm * 8));
    if (m)
        edge_map_kernel<<<grid_of(m), 256, 0, st>>>(dsrc.as<long long>(), ddst.as<long long>(), m,
                                                     keys.as<unsigned long long>(), vals.as<int32_t>(), cap - 1,
                                                     undirected, packed.as<unsigned long long>(), err.as<int32_t>());
    SU_CK(cudaGetLastError());
    int32_t herr = 0;
    SU_CK(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st));
    SU_CK(cudaStreamSynchronize(st));
    if (herr == 1) {
        *why = "an agent id appears twice";
        return SG_ERR_INVALID;
    }
    if (herr == 2) {
        *why = "an edge names an agent id that is not in the id list";
        return SG_ERR_BAD_CSR;
    }
    // sort (stable) and keep the first of each (src, dst)
    SU_CK(pos.get((size_t)mm * 4));
    SU_CK(sortk.get((size_t)mm * 8));
    SU_CK(sortv.get((size_t)mm * 4));
    if (mm) iota_kernel<<<grid_of(mm), 256, 0, st>>>(pos.as<uint32_t>(), mm);
    SU_CK(cudaGetLastError());
    size_t tbytes = 0, t2 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tbytes, packed.as<unsigned long long>(), sortk.as<unsigned long long>(),
                                    pos.as<uint32_t>(), sortv.as<uint32_t>(), (int)mm);
    cub::DeviceScan::ExclusiveSum(nullptr, t2, (int32_t *)nullptr, (int32_t *)nullptr, (int)std::max<long long>(mm, n + 1));
    tbytes = std::max(tbytes, t2);
    SU_CK(tmp.get(tbytes));
    if (mm)
        SU_CK(cub::DeviceRadixSort::SortPairs(tmp.p, tbytes, packed.as<unsigned long long>(),
                                              sortk.as<unsigned long long>(), pos.as<uint32_t>(),
                                              sortv.as<uint32_t>(), (int)mm, 0, 64, st));
    SU_CK(keep.get((size_t)mm * 4));
    SU_CK(at.get((size_t)(mm + 1) * 4));
    if (mm) first_of_run_kernel<<<grid_of(mm), 256, 0, st>>>(sortk.as<unsigned long long>(), mm, keep.as<int32_t>());
    SU_CK(cudaGetLastError());
    size_t sb = tbytes;
    if (mm)
        SU_CK(cub::DeviceScan::ExclusiveSum(tmp.p, sb, keep.as<int32_t>(), at.as<int32_t>(), (int)mm, st));
    int32_t last_keep = 0, last_at = 0;
    if (mm) {
        SU_CK(cudaMemcpyAsync(&last_keep, keep.as<int32_t>() + mm - 1, 4, cudaMemcpyDeviceToHost, st));
        SU_CK(cudaMemcpyAsync(&last_at, at.as<int32_t>() + mm - 1, 4, cudaMemcpyDeviceToHost, st));
    }
    SU_CK(cudaStreamSynchronize(st));
    const long long nnz = mm ? (long long)last_at + last_keep : 0;
    SU_CK(key2.get((size_t)nnz * 8));
    SU_CK(dst2.get((size_t)nnz * 4));
    if (mm)
        compact_kernel<<<grid_of(mm), 256, 0, st>>>(sortk.as<unsigned long long>(), sortv.as<uint32_t>(),
                                                    keep.as<int32_t>(), at.as<int32_t>(), mm, ordered,
                                                    key2.as<unsigned long long>(), dst2.as<uint32_t>());
    SU_CK(cudaGetLastError());
    // ordered rows: sort again by (src, first position); the neighbour rides along
    unsigned long long *final_keys = key2.as<unsigned long long>();
    if (ordered && nnz) {
        size_t need = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, need, key2.as<unsigned long long>(), sortk.as<unsigned long long>(),
                                        dst2.as<uint32_t>(), sortv.as<uint32_t>(), (int)nnz);
        if (need > tbytes) {
            Buf t3;
            SU_CK(t3.get(need));
            std::swap(tmp.p, t3.p);
            tbytes = need;
        }
        SU_CK(cub::DeviceRadixSort::SortPairs(tmp.p, need, key2.as<unsigned long long>(),
                                              sortk.as<unsigned long long>(), dst2.as<uint32_t>(),
                                              sortv.as<uint32_t>(), (int)nnz, 0, 64, st));
        final_keys = sortk.as<unsigned long long>();
    }
    // offsets and indices (the engine takes ownership of both arrays)
    int32_t *off = nullptr, *idx = nullptr;
    SU_CK(cudaMalloc(&off, (size_t)(n + 1) * 4));
    if (cudaMalloc(&idx, (size_t)std::max<long long>(nnz, 1) * 4) != cudaSuccess) {
        cudaFree(off);
        *why = "cudaMalloc of the CSR indices failed";
        return SG_ERR_CUDA;
    }
    *d_off = off;
    *d_idx = idx;
    SU_CK(cnt.get((size_t)(n + 1) * 4));
    SU_CK(cudaMemsetAsync(cnt.p, 0, (size_t)(n + 1) * 4, st));
    if (nnz) row_count_kernel<<<grid_of(nnz), 256, 0, st>>>(final_keys, nnz, cnt.as<int32_t>());
    SU_CK(cudaGetLastError());
    sb = tbytes;
    SU_CK(cub::DeviceScan::ExclusiveSum(tmp.p, sb, cnt.as<int32_t>(), off, (int)(n + 1), st));
    if (nnz) {
        if (ordered)
            SU_CK(cudaMemcpyAsync(idx, sortv.p, (size_t)nnz * 4, cudaMemcpyDeviceToDevice, st));
        else
            low_word_kernel<<<grid_of(nnz), 256, 0, st>>>(final_keys, nnz, idx);
    }
    SU_CK(cudaGetLastError());
    SU_CK(cudaStreamSynchronize(st));
    *nnz_out = nnz;
    return SG_OK;
}
