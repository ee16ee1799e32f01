// sg_philox.h -- SAGESim's Philox-2x32-10 stream, for host and device code.
//
// Counter layout of sagesim/math_utils.py:106-189 (rand_uniform_philox):
//   c0 = (tick * 1000003 + salt) mod 2^32, c1 = logical id mod 2^32,
//   key = seed mod 2^32, ten rounds (c0, c1) <- (hi(M*c0) ^ key ^ c1, lo(M*c0))
//   with key += 0x9E3779B9 after rounds 1..9, result k = c0 mod 2^23 and
//   u = k / 2^23.
// M is the multiplier the reference code uses, 3529668003 = 0xD26275A3
// (math_utils.py:111); its comment at math_utils.py:81 names 0xD256D193, but
// the arithmetic defines the stream.
//
// Because (a + b) mod 2^32 is a ring homomorphism, c0 for salt s is
// c0base + s with c0base = (uint32)(tick * 1000003); kernels hoist c0base per
// tick and the key/c1 per agent.
#pragma once
#if defined(__CUDACC_RTC__)
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef int int32_t;
#else
#include <stdint.h>
#endif

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define SG_HD __host__ __device__ __forceinline__
#else
#define SG_HD inline
#endif

#define SG_PHILOX_M 0xD26275A3u
#define SG_PHILOX_W 0x9E3779B9u

// Returns the 23-bit Philox integer for counter (c0, c1) and key. Each round is
// one 32x32->64-bit multiply (both halves at once) and a three-way xor.
SG_HD uint32_t sg_philox_k23(uint32_t c0, uint32_t c1, uint32_t key)
{
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        const uint64_t p = (uint64_t)c0 * SG_PHILOX_M;
        c0 = (uint32_t)(p >> 32) ^ key ^ c1;
        c1 = (uint32_t)p;
        if (r < 9) key += SG_PHILOX_W;
    }
    return c0 & 0x7FFFFFu;
}

// Round keys key + r * W (r = 0..9) of one seed, computed once and reused by
// every draw of a kernel that draws many times for the same seed.
struct SgPhiloxKeys {
    uint32_t k[10];
};

SG_HD SgPhiloxKeys sg_philox_keys(uint32_t key)
{
    SgPhiloxKeys ks;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) ks.k[r] = key + (uint32_t)r * SG_PHILOX_W;
    return ks;
}

SG_HD uint32_t sg_philox_k23_keys(uint32_t c0, uint32_t c1, const SgPhiloxKeys &ks)
{
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        const uint64_t p = (uint64_t)c0 * SG_PHILOX_M;
        c0 = (uint32_t)(p >> 32) ^ ks.k[r] ^ c1;
        c1 = (uint32_t)p;
    }
    return c0 & 0x7FFFFFu;
}

SG_HD uint32_t sg_c0base(int64_t tick)
{
    return (uint32_t)(uint64_t)(tick * 1000003LL);
}

#if !defined(__CUDACC_RTC__)
// Integer threshold K with (k / 2^23 < p) <=> (k < K) for a float64 p:
// k/2^23 < p <=> k < p*2^23 (exact scaling) <=> k < ceil(p*2^23).
inline uint32_t sg_threshold_host(double p)
{
    // ldexp-free: multiplying by 2^23 is exact for every finite double in range.
    const double x = p * 8388608.0;
    if (!(x > 0.0)) return 0u;
    if (x >= 8388608.0) return 8388608u;
    uint32_t k = (uint32_t)x;          // floor for x > 0
    if ((double)k < x) k += 1u;        // ceil
    return k;
}
#endif
