// strata.cu - deterministic training: a stratified schedule of the same per-rating update.
//
// Batch-Hogwild (sgd_update.cu) lets thousands of workers update shared rows without locks,
// so results vary from run to run.  With `deterministic` set, the shuffled ratings are
// bucketed into a G x G grid of blocks (user group u mod G, item group v mod G) and an epoch
// runs the G strata in a seeded random order: stratum s holds the blocks (a, (a + s) mod G)
// for a = 0 .. G-1, which share no user and no item, so G workers update them in parallel without any row in common and
// the result is the same on every run and equal to the serial restatement.  Within a block the
// ratings keep their input order (a stable sort).  The per-rating arithmetic is the update of
// singleGPU/sgd_k128_kernel_hogwild_warp32.h:85-99 exactly as the batch-Hogwild kernel does it
// (lane-partial fused multiply-adds, group butterfly, storage rounding, stochastic rounding
// keyed by the rating's position in the stratified array).
#include <cub/cub.cuh>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "cumf_sgd.h"
#include "device_common.cuh"
#include "internal.h"

namespace cumf {

namespace {

constexpr int kST = 256;  // threads per block of the stratum kernel

__global__ void block_key_kernel(const cumf_node *__restrict__ R, int64_t nnz, int G, uint32_t *keys,
                                 int64_t *idx, unsigned long long *counts) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const cumf_node x = R[i];
        const uint32_t key = ((uint32_t)x.u % (uint32_t)G) * (uint32_t)G + (uint32_t)x.v % (uint32_t)G;
        keys[i] = key;
        idx[i] = i;
        atomicAdd(&counts[key], 1ull);
    }
}

__global__ void gather_records_kernel(const cumf_node *__restrict__ R, const int64_t *__restrict__ idx, int64_t nnz,
                                      cumf_node *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = R[idx[i]];
}

// One worker (a group of L lanes) per block of the stratum; the block's ratings in order.
template <int K, int KIND, int L, bool SR>
__global__ void __launch_bounds__(kST) stratum_kernel(const cumf_node *__restrict__ R,
                                                      const unsigned long long *__restrict__ block_off, int G,
                                                      int stratum, void *Pv, void *Qv, uint32_t m, uint32_t n,
                                                      float lr, float lp, float lq, uint32_t round_key, int *status) {
    using C = Conv<KIND>;
    constexpr int ROW_WORDS = K * store_bytes(KIND) / 16;
    constexpr int NV = ROW_WORDS / L;
    static_assert(NV >= 1 && NV * L == ROW_WORDS, "lane split must cover the row");
    const int lane = threadIdx.x % L;
    const int a = (blockIdx.x * kST + threadIdx.x) / L;
    if (a >= G) return;
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
    const int b = (a + stratum) % G;
    const int blk = a * G + b;
    uint4 *const P = reinterpret_cast<uint4 *>(Pv) + lane * NV;
    uint4 *const Q = reinterpret_cast<uint4 *>(Qv) + lane * NV;
    const uint64_t pol = l2_policy(true, true);
    const unsigned long long i0 = block_off[blk], i1 = block_off[blk + 1];
    int bad = 0;
    if (i0 >= i1) return;
    // One-deep pipeline: the rows of rating i+1 are loaded while rating i is computed; when
    // rating i+1 reuses a row that rating i has just written, the fresh values are forwarded,
    // so the block's ratings are applied strictly in order.
    cumf_node x = R[i0];
    bool ok = ((uint32_t)x.u < m) & ((uint32_t)x.v < n);
    uint4 fp[NV], fq[NV];
#pragma unroll
    for (int w = 0; w < NV; ++w) {
        fp[w] = ok ? ld_row_hint(P + (uint64_t)(uint32_t)x.u * ROW_WORDS + w, pol) : make_uint4(0, 0, 0, 0);
        fq[w] = ok ? ld_row_hint(Q + (uint64_t)(uint32_t)x.v * ROW_WORDS + w, pol) : make_uint4(0, 0, 0, 0);
    }
    for (unsigned long long i = i0; i < i1; ++i) {
        const bool has_next = i + 1 < i1;
        const cumf_node xn = has_next ? R[i + 1] : x;
        const bool okn = has_next && ((uint32_t)xn.u < m) & ((uint32_t)xn.v < n);
        uint4 np[NV], nq[NV];
#pragma unroll
        for (int w = 0; w < NV; ++w) {
            np[w] = okn ? ld_row_hint(P + (uint64_t)(uint32_t)xn.u * ROW_WORDS + w, pol) : make_uint4(0, 0, 0, 0);
            nq[w] = okn ? ld_row_hint(Q + (uint64_t)(uint32_t)xn.v * ROW_WORDS + w, pol) : make_uint4(0, 0, 0, 0);
        }
        if (ok) {
            const uint32_t u = (uint32_t)x.u, v = (uint32_t)x.v;
            float sdot = 0.f;
#pragma unroll
            for (int w = 0; w < NV; ++w) {
#pragma unroll
                for (int h = 0; h < C::kPairs; ++h) {
                    const float2 pp = C::get(fp[w], h), qq = C::get(fq[w], h);
                    sdot = __fmaf_rn(pp.x, qq.x, sdot);
                    sdot = __fmaf_rn(pp.y, qq.y, sdot);
                }
            }
#pragma unroll
            for (int o = L / 2; o >= 1; o >>= 1) sdot += __shfl_xor_sync(gmask, sdot, o);
            const float err = x.r - sdot;
            const uint32_t key = SR ? (round_key ^ lowbias32((uint32_t)i)) : 0u;
            uint4 wp[NV], wq[NV];
#pragma unroll
            for (int w = 0; w < NV; ++w) {
#pragma unroll
                for (int h = 0; h < C::kPairs; ++h) {
                    const float2 pp = C::get(fp[w], h), qq = C::get(fq[w], h);
                    const float px = __fmaf_rn(lr, __fmaf_rn(err, qq.x, -__fmul_rn(lp, pp.x)), pp.x);
                    const float py = __fmaf_rn(lr, __fmaf_rn(err, qq.y, -__fmul_rn(lp, pp.y)), pp.y);
                    const float qx = __fmaf_rn(lr, __fmaf_rn(err, pp.x, -__fmul_rn(lq, qq.x)), qq.x);
                    const float qy = __fmaf_rn(lr, __fmaf_rn(err, pp.y, -__fmul_rn(lq, qq.y)), qq.y);
                    if (SR) {
                        const uint32_t pair = (uint32_t)(((lane * NV + w) * C::kPairs + h) * 2);
                        C::put_sr(wp[w], h, px, py, lowbias32(key + pair));
                        C::put_sr(wq[w], h, qx, qy, lowbias32(key + pair + 1u));
                    } else {
                        C::put(wp[w], h, px, py);
                        C::put(wq[w], h, qx, qy);
                    }
                }
            }
#pragma unroll
            for (int w = 0; w < NV; ++w) {
                st_row_hint(P + (uint64_t)u * ROW_WORDS + w, wp[w], pol);
                st_row_hint(Q + (uint64_t)v * ROW_WORDS + w, wq[w], pol);
            }
            if (okn && (uint32_t)xn.u == u) {
#pragma unroll
                for (int w = 0; w < NV; ++w) np[w] = wp[w];
            }
            if (okn && (uint32_t)xn.v == v) {
#pragma unroll
                for (int w = 0; w < NV; ++w) nq[w] = wq[w];
            }
        } else {
            bad = 1;
        }
#pragma unroll
        for (int w = 0; w < NV; ++w) {
            fp[w] = np[w];
            fq[w] = nq[w];
        }
        x = xn;
        ok = okn;
    }
    if (bad && status != nullptr && lane == 0) atomicExch(status, (int)CUMF_ERR_RANGE);
}

using StratumFn = void (*)(const cumf_node *, const unsigned long long *, int, int, void *, void *, uint32_t,
                           uint32_t, float, float, float, uint32_t, int *);

// One 16-byte word per lane (the update kernel's default layout).
template <int K>
StratumFn pick(int precision, int *lanes) {
    switch (precision) {
        case CUMF_FP16: *lanes = K * 2 / 16; return &stratum_kernel<K, kHalf, K * 2 / 16, false>;
        case CUMF_FP16_SR: *lanes = K * 2 / 16; return &stratum_kernel<K, kHalf, K * 2 / 16, true>;
        case CUMF_BF16: *lanes = K * 2 / 16; return &stratum_kernel<K, kBf16, K * 2 / 16, false>;
        case CUMF_BF16_SR: *lanes = K * 2 / 16; return &stratum_kernel<K, kBf16, K * 2 / 16, true>;
        default: *lanes = std::min(32, K * 4 / 16); return &stratum_kernel<K, kFloat, (K * 4 / 16 > 32 ? 32 : K * 4 / 16), false>;
    }
}

}  // namespace

// The strata of epoch ep in a seeded random order: Fisher-Yates over 0 .. G-1 drawing
// splitmix64(seed ^ tag, epoch, step) mod (step + 1).
void strata_order(uint64_t seed, int ep, int G, int *order) {
    for (int i = 0; i < G; ++i) order[i] = i;
    uint64_t h = splitmix64(seed ^ (0x5354ull << 48)) + (uint64_t)ep * 0x9E3779B97F4A7C15ull;
    for (int i = G - 1; i > 0; --i) {
        h = splitmix64(h);
        const int j = (int)(h % (uint64_t)(i + 1));
        const int t = order[i];
        order[i] = order[j];
        order[j] = t;
    }
}

int strata_groups(int64_t nnz, int requested) {
    if (requested > 1) return requested;
    // About 24 ratings per block: G^2 blocks, G workers per stratum.
    const double g = sqrt((double)std::max<int64_t>(1, nnz) / 24.0);
    return (int)std::max(1.0, std::min(2048.0, std::floor(g)));
}

int strata_layout(const cumf_node *d_R, int64_t nnz, int G, cumf_node *d_out, unsigned long long *d_block_off,
                  cudaStream_t s) {
    if (G < 1 || (int64_t)G * G > (1ll << 26)) return fail(CUMF_ERR_ARG, "strata: group count out of range");
    const int64_t blocks = (int64_t)G * G;
    struct Buf {
        void *p = nullptr;
        ~Buf() {
            if (p) cudaFree(p);
        }
    } keys, keys2, idx, idx2, counts, tmp;
    const size_t n = (size_t)std::max<int64_t>(1, nnz);
    CUMF_CUDA(cudaMalloc(&keys.p, n * 4));
    CUMF_CUDA(cudaMalloc(&keys2.p, n * 4));
    CUMF_CUDA(cudaMalloc(&idx.p, n * 8));
    CUMF_CUDA(cudaMalloc(&idx2.p, n * 8));
    CUMF_CUDA(cudaMalloc(&counts.p, (size_t)(blocks + 1) * 8));
    unsigned long long *cnt = static_cast<unsigned long long *>(counts.p);
    CUMF_CUDA(cudaMemsetAsync(cnt, 0, (size_t)(blocks + 1) * 8, s));
    const int grid = (int)std::min<int64_t>(65535, (nnz + 255) / 256 + 1);
    block_key_kernel<<<grid, 256, 0, s>>>(d_R, nnz, G, static_cast<uint32_t *>(keys.p),
                                          static_cast<int64_t *>(idx.p), cnt);
    CUMF_CUDA(cudaGetLastError());
    // Stable sort by block (keeps the input order inside a block), then block offsets.
    int end_bit = 1;
    while (end_bit < 32 && ((uint64_t)1 << end_bit) < (uint64_t)blocks) ++end_bit;
    size_t tb = 0;
    CUMF_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, static_cast<uint32_t *>(keys.p),
                                              static_cast<uint32_t *>(keys2.p), static_cast<int64_t *>(idx.p),
                                              static_cast<int64_t *>(idx2.p), nnz, 0, end_bit, s));
    size_t tb2 = 0;
    CUMF_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb2, cnt, d_block_off, blocks + 1, s));
    CUMF_CUDA(cudaMalloc(&tmp.p, std::max(tb, tb2) + 16));
    CUMF_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, static_cast<uint32_t *>(keys.p),
                                              static_cast<uint32_t *>(keys2.p), static_cast<int64_t *>(idx.p),
                                              static_cast<int64_t *>(idx2.p), nnz, 0, end_bit, s));
    CUMF_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb2, cnt, d_block_off, blocks + 1, s));
    gather_records_kernel<<<grid, 256, 0, s>>>(d_R, static_cast<const int64_t *>(idx2.p), nnz, d_out);
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(cudaStreamSynchronize(s));  // the scratch above is freed on return
    return CUMF_OK;
}

int strata_epochs(const cumf_node *d_S, const unsigned long long *d_block_off, int G, void *d_P, int32_t m,
                  void *d_Q, int32_t n, int k, int precision, const float *h_lr, int first_epoch, int n_epochs,
                  float lambda_p, float lambda_q, uint64_t seed, int *d_status, cudaStream_t s) {
    int lanes = 0;
    StratumFn fn = nullptr;
    switch (k) {
        case 32: fn = pick<32>(precision, &lanes); break;
        case 64: fn = pick<64>(precision, &lanes); break;
        case 128: fn = pick<128>(precision, &lanes); break;
        case 256: fn = pick<256>(precision, &lanes); break;
        default: return fail(CUMF_ERR_ARG, "strata: k must be 32, 64, 128 or 256");
    }
    const int groups_per_block = kST / lanes;
    const int blocks = (G + groups_per_block - 1) / groups_per_block;
    std::vector<int> order(G);
    for (int ep = first_epoch; ep < first_epoch + n_epochs; ++ep) {
        const uint32_t round_key = (uint32_t)(splitmix64(seed ^ (kTagRound << 48)) + (uint64_t)ep);
        strata_order(seed, ep, G, order.data());
        for (int j = 0; j < G; ++j)
            fn<<<blocks, kST, 0, s>>>(d_S, d_block_off, G, order[j], d_P, d_Q, (uint32_t)m, (uint32_t)n, h_lr[ep],
                                      lambda_p, lambda_q, round_key, d_status);
        CUMF_CUDA(cudaGetLastError());
    }
    return CUMF_OK;
}

}  // namespace cumf

using namespace cumf;

extern "C" int cumf_dev_strata_layout(const cumf_node *d_R, int64_t nnz, int groups, cumf_node *d_out,
                                      unsigned long long *d_block_off, void *stream) {
    if (nnz < 0 || (nnz > 0 && (!d_R || !d_out)) || !d_block_off) return fail(CUMF_ERR_ARG, "strata_layout: bad arguments");
    return strata_layout(d_R, nnz, groups, d_out, d_block_off, static_cast<cudaStream_t>(stream));
}

extern "C" int cumf_dev_strata_epochs(const cumf_node *d_S, const unsigned long long *d_block_off, int groups,
                                      void *d_P, int32_t m, void *d_Q, int32_t n, int k, int precision,
                                      const float *h_lr, int first_epoch, int n_epochs, float lambda_p,
                                      float lambda_q, uint64_t seed, int *d_status, void *stream) {
    if (groups < 1 || !d_block_off || !d_P || !d_Q || !h_lr || first_epoch < 0 || n_epochs < 0 || m < 1 || n < 1)
        return fail(CUMF_ERR_ARG, "strata_epochs: bad arguments");
    if (precision < CUMF_FP16 || precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    return strata_epochs(d_S, d_block_off, groups, d_P, m, d_Q, n, k, precision, h_lr, first_epoch, n_epochs,
                         lambda_p, lambda_q, seed, d_status, static_cast<cudaStream_t>(stream));
}
