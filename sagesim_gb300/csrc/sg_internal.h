// sg_internal.h -- shared host-side helpers of the engine translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/sagesim_gb300.h"
#include "sg_kernels.h"

// Owning device allocation.
struct SgDev {
    void *p = nullptr;
    size_t bytes = 0;
    SgDev() = default;
    SgDev(const SgDev &) = delete;
    SgDev &operator=(const SgDev &) = delete;
    SgDev(SgDev &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    SgDev &operator=(SgDev &&o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            bytes = o.bytes;
            o.p = nullptr;
            o.bytes = 0;
        }
        return *this;
    }
    ~SgDev() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // Grows to at least `b` bytes (contents not kept).
    cudaError_t reserve(size_t b)
    {
        if (b <= bytes && p) return cudaSuccess;
        release();
        if (b == 0) b = 16;
        cudaError_t err = cudaMalloc(&p, b);
        if (err != cudaSuccess) {
            p = nullptr;
            return err;
        }
        bytes = b;
        return cudaSuccess;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// Time accumulated per kernel kind when profiling is on.
struct SgProfKind {
    std::string name;
    int64_t launches = 0;
    double total_ms = 0.0;
};

struct SgProfiler {
    bool on = false;
    std::vector<SgProfKind> kinds;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> pool;

    int kind(const char *name)
    {
        for (size_t i = 0; i < kinds.size(); ++i)
            if (kinds[i].name == name) return (int)i;
        kinds.push_back(SgProfKind{name, 0, 0.0});
        return (int)kinds.size() - 1;
    }
    cudaEvent_t get()
    {
        if (!pool.empty()) {
            cudaEvent_t ev = pool.back();
            pool.pop_back();
            return ev;
        }
        cudaEvent_t ev = nullptr;
        cudaEventCreate(&ev);
        return ev;
    }
    // Records the start event of a launch of `k` on `st`; returns a token.
    size_t begin(int k, cudaStream_t st)
    {
        cudaEvent_t a = get(), b = get();
        cudaEventRecord(a, st);
        pending.push_back({k, {a, b}});
        return pending.size() - 1;
    }
    void end(size_t token, cudaStream_t st) { cudaEventRecord(pending[token].second.second, st); }
    // Call after the stream is synchronized.
    void collect()
    {
        for (auto &pe : pending) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
            kinds[pe.first].launches += 1;
            kinds[pe.first].total_ms += ms;
            pool.push_back(pe.second.first);
            pool.push_back(pe.second.second);
        }
        pending.clear();
    }
    void destroy()
    {
        collect();
        for (cudaEvent_t ev : pool) cudaEventDestroy(ev);
        pool.clear();
    }
};

inline int sg_sm_count(int device)
{
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0)
        v = 152;
    return v;
}

// Tile list over [begin, end) for segment `seg`, SG_TILE agents per tile.
inline void sg_append_tiles(std::vector<SgTile> &tiles, int32_t seg, int64_t begin, int64_t end)
{
    for (int64_t b = begin; b < end; b += SG_TILE) {
        const int64_t e = b + SG_TILE < end ? b + SG_TILE : end;
        tiles.push_back(SgTile{seg, (int32_t)b, (int32_t)e, 0});
    }
}

// CSR validation shared by the engine and the batch (host arrays).
// Returns an empty string when valid.
std::string sg_check_csr(const int32_t *off, int64_t n, const int32_t *idx, int64_t nnz);
