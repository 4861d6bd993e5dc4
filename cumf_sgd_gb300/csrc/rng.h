// rng.h - counter-based random numbers shared by host and device code.
//
// The reference draws batch starts with cuRAND XORWOW states seeded from clock()
// (singleGPU/sgd_kernel.cu:22-26, singleGPU/sgd_k128_kernel_hogwild_warp32.h:42-47) and
// factor init values the same way (singleGPU/sgd.cu:491-514), so its sample order cannot be
// reproduced.  Here every draw is a pure function of (seed, counters), which makes a run
// repeatable and lets a CPU restatement replay the exact sample order.
//
// Mixer: SplitMix64 finalizer (G. Steele, D. Lea, C. Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014), the published 64-bit mix with constants
// 0x9E3779B97F4A7C15 / 0xBF58476D1CE4E5B9 / 0x94D049BB133111EB.
// Per-element stochastic-rounding bits use the 32-bit "lowbias32" integer hash
// (C. Wellons, "Prospecting for hash functions", 2018).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CUMF_HD __host__ __device__ __forceinline__
#else
#define CUMF_HD inline
#endif

namespace cumf {

CUMF_HD uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

CUMF_HD uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// High 64 bits of a*b: maps a uniform 64-bit word onto [0, n).
CUMF_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Stream keys: distinct constants keep the init, sample and rounding streams apart.
constexpr uint64_t kTagSample = 0x5341u;  // batch starts
constexpr uint64_t kTagRound = 0x5352u;   // stochastic rounding
// Factor init tags passed by the caller: P = 1, Q = 2.

// Start record of batch `batch` of worker `worker` in epoch `epoch`: uniform on [0, nnz).
CUMF_HD uint64_t batch_start(uint64_t seed, uint32_t epoch, uint32_t worker, uint32_t batch,
                             uint64_t nnz) {
    uint64_t h = splitmix64(seed ^ (kTagSample << 48));
    h = splitmix64(h + epoch);
    h = splitmix64(h + worker);
    h = splitmix64(h + batch);
    return mulhi64(h, nnz);
}

// Key of a factor-init stream (tag 1 = P, 2 = Q).
CUMF_HD uint64_t init_key(uint64_t seed, uint32_t tag) {
    return splitmix64(splitmix64(seed) + tag);
}

// Uniform on (0, 1] with 24 random bits, like curand_uniform's range (sgd.cu:512).
CUMF_HD float init_uniform(uint64_t key, uint64_t index) {
    uint64_t h = splitmix64(key ^ index);
    return (float)((h >> 40) + 1) * (1.0f / 16777216.0f);
}

}  // namespace cumf
