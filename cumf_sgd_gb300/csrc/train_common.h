// train_common.h - host helpers shared by the training drivers (modes A, B and C).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "cumf_sgd.h"
#include "glibc_shuffle.h"
#include "internal.h"

namespace cumf {

// RAII device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t b) {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = b;
        return cudaMalloc(&p, b ? b : 16);
    }
    template <typename T>
    T *as() const { return reinterpret_cast<T *>(p); }
};

struct Stream {
    cudaStream_t s = nullptr;
    ~Stream() {
        if (s) cudaStreamDestroy(s);
    }
};

struct Event {
    cudaEvent_t e = nullptr;
    ~Event() {
        if (e) cudaEventDestroy(e);
    }
    cudaError_t create() { return cudaEventCreate(&e); }
};

inline double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

inline bool valid_k(int k) { return k == 32 || k == 64 || k == 128 || k == 256; }

inline int check_params(const cumf_params *p) {
    if (!p) return fail(CUMF_ERR_ARG, "params is NULL");
    if (!valid_k(p->k)) return fail(CUMF_ERR_ARG, "k must be 32, 64, 128 or 256 (got " + std::to_string(p->k) + ")");
    if (p->num_workers < 0) return fail(CUMF_ERR_ARG, "num_workers must be >= 0 (0 = automatic)");
    if (p->num_iters < 0) return fail(CUMF_ERR_ARG, "num_iters must be >= 0");
    if (p->u_grid < 1 || p->v_grid < 1 || p->x_grid < 1 || p->y_grid < 1)
        return fail(CUMF_ERR_ARG, "grid sizes must be positive");
    if (p->precision < CUMF_FP16 || p->precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    if (p->deterministic < 0 || p->deterministic > 4096)
        return fail(CUMF_ERR_ARG, "deterministic must be 0 (batch-Hogwild), 1 (automatic grid) or a grid of 2..4096");
    if (p->deterministic > 0 && p->u_grid * p->v_grid != 1)
        return fail(CUMF_ERR_ARG, "the deterministic schedule needs u = v = 1 (the whole problem in HBM)");
    if (p->deterministic > 0 && p->tail_epochs > 0)
        return fail(CUMF_ERR_ARG, "the deterministic schedule has no fold-in epochs");
    if (p->lanes != 0 && !lanes_supported(p->k, p->precision, p->lanes))
        return fail(CUMF_ERR_ARG, "unsupported lane count " + std::to_string(p->lanes) + " for k=" + std::to_string(p->k));
    return CUMF_OK;
}

inline int select_device(int gpu) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return fail(CUMF_ERR_NODEVICE, "no CUDA device visible");
    }
    int dev = gpu % count;  // main.cpp:292-294
    if (dev < 0) dev += count;
    CUMF_CUDA(cudaSetDevice(dev));
    return CUMF_OK;
}

// Host-side fp16/bf16 -> fp32 (exact widening), for the streamed modes' export.
inline float half_bits_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t exp = (h >> 10) & 0x1f, man = h & 0x3ffu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {  // subnormal: renormalise
            int e = -1;
            uint32_t mm = man;
            do {
                mm <<= 1;
                ++e;
            } while ((mm & 0x400u) == 0);
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((mm & 0x3ffu) << 13);
        }
    } else if (exp == 0x1f) {
        bits = sign | 0x7f800000u | (man << 13);
    } else {
        bits = sign | ((exp + 127 - 15) << 23) | (man << 13);
    }
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

inline float store_to_float(const void *base, int64_t idx, int precision) {
    if (precision == CUMF_FP32) return reinterpret_cast<const float *>(base)[idx];
    const uint16_t h = reinterpret_cast<const uint16_t *>(base)[idx];
    if (precision == CUMF_BF16 || precision == CUMF_BF16_SR) {
        const uint32_t bits = (uint32_t)h << 16;
        float f;
        memcpy(&f, &bits, 4);
        return f;
    }
    return half_bits_to_float(h);
}

struct Prepared {
    float ave = 0, std_dev = 0, scale = 1;
    std::vector<int32_t> pmap, qmap;
    GlibcRand rng{0};
};

// Rating statistics -> float mean/std and the scale max(1e-4, std) (sgd.cu:78-96, 648-649).
inline void finish_stats(double sum, double sum2, int64_t nnz, Prepared &pr) {
    double ex = nnz ? sum / (double)nnz : 0.0;
    double ex2 = nnz ? sum2 / (double)nnz : 0.0;
    pr.ave = (float)ex;
    pr.std_dev = (float)sqrt(ex2 - ex * ex);
    pr.scale = std::max(1e-4f, pr.std_dev);
}

// gen_random_map x2 (sgd.cu:656-657): both maps restart the glibc stream from the same seed
// (srand(time(NULL)) is called inside each).  The stream continues after the q map into the
// block shuffles of modes B/C (sgd_kernel.cu:263-267, 411-431).
inline void make_maps(uint32_t seed, int32_t m, int32_t n, Prepared &pr) {
    pr.pmap.resize(m);
    pr.qmap.resize(n);
    GlibcRand r1(seed);
    for (int32_t i = 0; i < m; ++i) pr.pmap[i] = i;
    glibc_random_shuffle(pr.pmap.data(), m, r1);
    pr.rng.reseed(seed);
    for (int32_t i = 0; i < n; ++i) pr.qmap[i] = i;
    glibc_random_shuffle(pr.qmap.data(), n, pr.rng);
}

}  // namespace cumf
