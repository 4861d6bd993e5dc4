// prep.cu - data preparation, factor init, fp32 export and the RMSE evaluator.
//
// Reference counterparts:
//   init_factors    random_init / init_feature      singleGPU/sgd.cu:497-546
//   rating_stats    collect_data                    singleGPU/sgd.cu:78-96
//   shuffle_scale   shuffle_problem + scale_problem singleGPU/sgd.cu:126-134, 98-124
//   export          transform_half + scale_model + shuffle_model
//                                                   singleGPU/sgd_kernel.cu:29-68,
//                                                   singleGPU/sgd.cu:593-635
//   rmse            calc_rmse / mf_predict          test/mf.cpp:3794-3839
// All are HBM-streaming kernels (grid-stride, coalesced); the reductions are two-pass with a
// fixed grid so results do not depend on scheduling.
#include <cuda_runtime.h>
#include <algorithm>
#include <math.h>
#include <stdint.h>

#include "device_common.cuh"
#include "internal.h"

namespace cumf {

namespace {

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 1024;  // fixed grid of the two-pass reductions

template <int KIND>
__global__ void init_kernel(void *out, uint64_t count, int k, uint64_t key, uint64_t offset) {
    using S = Scalar<KIND>;
    typename S::T *o = reinterpret_cast<typename S::T *>(out);
    // (float)sqrt(1.0/k), the reference's scale (sgd.cu:519).
    const float scale = (float)sqrt(1.0 / (double)k);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        o[i] = S::from_float(__fmul_rn(init_uniform(key, offset + i), scale));
    }
}

__device__ __forceinline__ double block_sum(double x, double *sh) {
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = x;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
    __syncthreads();
    return t;  // valid in thread 0
}

__global__ void stats_kernel(const cumf_node *R, uint64_t nnz, double *part) {
    __shared__ double sh[2][kThreads / 32];
    double s = 0.0, s2 = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nnz;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const double r = (double)R[i].r;
        s += r;
        s2 += r * r;
    }
    const double a = block_sum(s, sh[0]);
    const double b = block_sum(s2, sh[1]);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// Sums `count` pairs of partials in index order (deterministic).
__global__ void sum_pairs_kernel(const double *part, int count, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < count; ++i) {
            a += part[2 * i];
            b += part[2 * i + 1];
        }
        out[0] = a;
        out[1] = b;
    }
}

__global__ void shuffle_scale_kernel(const cumf_node *in, cumf_node *out, uint64_t nnz,
                                     const int32_t *pmap, uint32_t m, const int32_t *qmap,
                                     uint32_t n, float scale, int *status) {
    int bad = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nnz;
         i += (uint64_t)gridDim.x * blockDim.x) {
        cumf_node x = in[i];
        const uint32_t u = (uint32_t)x.u, v = (uint32_t)x.v;
        if (u < m && v < n) {
            x.u = pmap ? pmap[u] : x.u;
            x.v = qmap ? qmap[v] : x.v;
        } else {
            bad = 1;
        }
        x.r = __fmul_rn(x.r, scale);
        out[i] = x;
    }
    if (bad && status) atomicExch(status, (int)CUMF_ERR_RANGE);
}

template <int KIND>
__global__ void export_kernel(const void *in, const int32_t *map, uint64_t rows, int k,
                              float factor, float *out) {
    using S = Scalar<KIND>;
    const typename S::T *src = reinterpret_cast<const typename S::T *>(in);
    const uint64_t count = rows * (uint64_t)k;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t o = i / (uint64_t)k, j = i - o * (uint64_t)k;
        const uint64_t srow = map ? (uint64_t)(uint32_t)map[o] : o;
        out[i] = __fmul_rn(S::to_float(src[srow * (uint64_t)k + j]), factor);
    }
}

// dst[map[o]] = storage(src[o] / factor) for o < rows: the inverse of the export.
template <int KIND>
__global__ void import_kernel(const float *src, const int32_t *map, uint64_t rows, int k, float factor, void *dst) {
    using S = Scalar<KIND>;
    typename S::T *d = reinterpret_cast<typename S::T *>(dst);
    const uint64_t count = rows * (uint64_t)k;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t o = i / (uint64_t)k, j = i - o * (uint64_t)k;
        const uint64_t drow = map ? (uint64_t)(uint32_t)map[o] : o;
        d[drow * (uint64_t)k + j] = S::from_float(__fdiv_rn(src[i], factor));
    }
}

// Eight lanes per rating; float dot in fp32, squared error rounded to fp32 and summed in
// fp64 as calc_rmse does (`mf_float e = r - z; loss += e*e;`, mf.cpp:3831-3834).
constexpr int kRmseLanes = 8;

__global__ void rmse_kernel(const cumf_node *R, uint64_t nnz, const float *P, uint32_t m,
                            const float *Q, uint32_t n, int k, float b, double *part) {
    __shared__ double sh[kThreads / 32];
    const int lane = threadIdx.x % kRmseLanes;
    const uint64_t group = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / kRmseLanes;
    const uint64_t groups = (uint64_t)gridDim.x * blockDim.x / kRmseLanes;
    const unsigned gmask = 0xffu << ((threadIdx.x & 31) & ~(kRmseLanes - 1));
    double acc = 0.0;
    for (uint64_t i = group; i < nnz; i += groups) {
        const cumf_node x = R[i];
        const uint32_t u = (uint32_t)x.u, v = (uint32_t)x.v;
        float z;
        if (u < m && v < n) {
            const float *p = P + (uint64_t)u * k;
            const float *q = Q + (uint64_t)v * k;
            float s = 0.f;
            if ((k & 3) == 0) {
                const float4 *p4 = reinterpret_cast<const float4 *>(p);
                const float4 *q4 = reinterpret_cast<const float4 *>(q);
                for (int c = lane; c < (k >> 2); c += kRmseLanes) {
                    const float4 a = __ldg(p4 + c), bq = __ldg(q4 + c);
                    s = __fmaf_rn(a.x, bq.x, s);
                    s = __fmaf_rn(a.y, bq.y, s);
                    s = __fmaf_rn(a.z, bq.z, s);
                    s = __fmaf_rn(a.w, bq.w, s);
                }
            } else {
                for (int c = lane; c < k; c += kRmseLanes) s = __fmaf_rn(__ldg(p + c), __ldg(q + c), s);
            }
            for (int o = kRmseLanes / 2; o >= 1; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
            z = isnan(s) ? b : s;
        } else {
            z = b;
        }
        if (lane == 0) {
            const float e = x.r - z;
            acc += (double)__fmul_rn(e, e);
        }
    }
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Sum of `count` partials in a fixed order (one block of kSumThreads): thread t adds
// part[t], part[t + kSumThreads], ... in index order, then a fixed tree over the threads.
// The same count always gives the same bits.
constexpr int kSumThreads = 256;
__global__ void __launch_bounds__(kSumThreads) sum_kernel(const double *part, int count, double *out) {
    __shared__ double sh[kSumThreads];
    double a = 0.0;
    for (int i = threadIdx.x; i < count; i += kSumThreads) a += part[i];
    sh[threadIdx.x] = a;
    __syncthreads();
#pragma unroll
    for (int w = kSumThreads / 2; w >= 1; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sh[0];
}

int grid_for(uint64_t items, int per_thread = 1) {
    uint64_t blocks = (items + (uint64_t)kThreads * per_thread - 1) / ((uint64_t)kThreads * per_thread);
    if (blocks < 1) blocks = 1;
    if (blocks > 152ull * 32) blocks = 152ull * 32;
    return (int)blocks;
}

// Order-independent 64-bit digest of a byte buffer (a multiple of 4 bytes): the sum of
// splitmix64(word, index) over its 32-bit words.
__global__ void digest_kernel(const uint32_t *w, uint64_t nwords, unsigned long long *out) {
    unsigned long long acc = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nwords; i += (uint64_t)gridDim.x * blockDim.x)
        acc += splitmix64(((uint64_t)__ldg(w + i) << 32) ^ (i * 0x9E3779B97F4A7C15ull));
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// `passes` copies of a[0..n16) to b within one launch, loads through L2 only (ld.global.cg),
// each thread on the same 16-byte words every pass: with a and b small enough, every pass
// after the first is served by L2.
__global__ void copy_passes_kernel(const uint4 *__restrict__ a, uint4 *__restrict__ b, uint64_t n16, int passes) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (int p = 0; p < passes; ++p) {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += stride) {
            uint4 v = __ldcg(a + i);
            v.x += (uint32_t)p;  // keeps every pass's copy live
            b[i] = v;
        }
    }
}

}  // namespace

cudaError_t launch_digest(const void *d, uint64_t bytes, unsigned long long *d_out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || bytes < 4) return e;
    const uint64_t words = bytes / 4;
    digest_kernel<<<grid_for(words, 8), kThreads, 0, s>>>(static_cast<const uint32_t *>(d), words, d_out);
    return cudaGetLastError();
}

cudaError_t launch_init_factors(void *d, int64_t rows, int k, int precision, uint64_t seed,
                                uint32_t tag, cudaStream_t s, uint64_t index_offset) {
    const uint64_t count = (uint64_t)rows * (uint64_t)k;
    if (count == 0) return cudaSuccess;
    const uint64_t key = init_key(seed, tag);
    const int g = grid_for(count, 4);
    switch (store_of_precision(precision)) {
        case kHalf: init_kernel<kHalf><<<g, kThreads, 0, s>>>(d, count, k, key, index_offset); break;
        case kBf16: init_kernel<kBf16><<<g, kThreads, 0, s>>>(d, count, k, key, index_offset); break;
        default: init_kernel<kFloat><<<g, kThreads, 0, s>>>(d, count, k, key, index_offset); break;
    }
    return cudaGetLastError();
}

int stats_blocks(int64_t nnz) {
    (void)nnz;
    return kReduceBlocks;
}

cudaError_t launch_rating_stats(const cumf_node *d_R, int64_t nnz, double *d_part,
                                double *d_out2, cudaStream_t s) {
    stats_kernel<<<kReduceBlocks, kThreads, 0, s>>>(d_R, (uint64_t)nnz, d_part);
    sum_pairs_kernel<<<1, 32, 0, s>>>(d_part, kReduceBlocks, d_out2);
    return cudaGetLastError();
}

cudaError_t launch_shuffle_scale(const cumf_node *in, cumf_node *out, int64_t nnz,
                                 const int32_t *pmap, int32_t m, const int32_t *qmap,
                                 int32_t n, float scale, int *d_status, cudaStream_t s) {
    if (nnz <= 0) return cudaSuccess;
    shuffle_scale_kernel<<<grid_for((uint64_t)nnz, 4), kThreads, 0, s>>>(
        in, out, (uint64_t)nnz, pmap, (uint32_t)m, qmap, (uint32_t)n, scale, d_status);
    return cudaGetLastError();
}

cudaError_t launch_export(const void *in, int precision, const int32_t *map, int64_t rows,
                          int k, float factor, float *out, cudaStream_t s) {
    const uint64_t count = (uint64_t)rows * (uint64_t)k;
    if (count == 0) return cudaSuccess;
    const int g = grid_for(count, 4);
    switch (store_of_precision(precision)) {
        case kHalf: export_kernel<kHalf><<<g, kThreads, 0, s>>>(in, map, rows, k, factor, out); break;
        case kBf16: export_kernel<kBf16><<<g, kThreads, 0, s>>>(in, map, rows, k, factor, out); break;
        default: export_kernel<kFloat><<<g, kThreads, 0, s>>>(in, map, rows, k, factor, out); break;
    }
    return cudaGetLastError();
}

int rmse_blocks(int64_t nnz) {
    (void)nnz;
    return kReduceBlocks;
}

cudaError_t launch_rmse(const cumf_node *d_R, int64_t nnz, const float *P, int32_t m,
                        const float *Q, int32_t n, int k, float b, double *d_part,
                        double *d_sum, cudaStream_t s) {
    rmse_kernel<<<kReduceBlocks, kThreads, 0, s>>>(d_R, (uint64_t)nnz, P, (uint32_t)m, Q,
                                                   (uint32_t)n, k, b, d_part);
    sum_kernel<<<1, kSumThreads, 0, s>>>(d_part, kReduceBlocks, d_sum);
    return cudaGetLastError();
}

cudaError_t launch_import(const float *src, const int32_t *map, int64_t rows, int k, float factor, void *dst,
                          int precision, cudaStream_t s) {
    const uint64_t count = (uint64_t)rows * (uint64_t)k;
    if (count == 0) return cudaSuccess;
    const int g = grid_for(count, 4);
    switch (store_of_precision(precision)) {
        case kHalf: import_kernel<kHalf><<<g, kThreads, 0, s>>>(src, map, rows, k, factor, dst); break;
        case kBf16: import_kernel<kBf16><<<g, kThreads, 0, s>>>(src, map, rows, k, factor, dst); break;
        default: import_kernel<kFloat><<<g, kThreads, 0, s>>>(src, map, rows, k, factor, dst); break;
    }
    return cudaGetLastError();
}

// Forces the (lazily loaded) evaluator kernels of launch_rmse_grid onto the current device
// without launching them: CUDA's lazy module loading would otherwise load them, and allocate
// for their code, at the first launch.
cudaError_t load_rmse_kernels() {
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, rmse_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, sum_kernel);
    return e;
}

cudaError_t launch_rmse_grid(const cumf_node *d_R, int64_t nnz, const float *P, int32_t m,
                             const float *Q, int32_t n, int k, float b, int blocks,
                             double *d_part, double *d_sum, cudaStream_t s) {
    rmse_kernel<<<blocks, kThreads, 0, s>>>(d_R, (uint64_t)nnz, P, (uint32_t)m, Q, (uint32_t)n, k, b, d_part);
    sum_kernel<<<1, kSumThreads, 0, s>>>(d_part, blocks, d_sum);
    return cudaGetLastError();
}

}  // namespace cumf

extern "C" int cumf_probe_copy_bandwidth(int64_t bytes, int passes, double *gbs, void *stream) {
    using namespace cumf;
    if (bytes < 16 || passes < 1 || !gbs) return fail(CUMF_ERR_ARG, "probe_copy_bandwidth: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t n16 = (uint64_t)bytes / 16;
    void *buf = nullptr;
    CUMF_CUDA(cudaMalloc(&buf, n16 * 32));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMemsetAsync(buf, 1, n16 * 32, s);
    const uint4 *a = static_cast<const uint4 *>(buf);
    uint4 *b = static_cast<uint4 *>(buf) + n16;
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::max(1, sms) * 8;
    if (e == cudaSuccess) copy_passes_kernel<<<grid, 256, 0, s>>>(a, b, n16, 2);  // warm: both buffers in cache
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) copy_passes_kernel<<<grid, 256, 0, s>>>(a, b, n16, passes);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "probe_copy_bandwidth");
    *gbs = ms > 0 ? 2.0 * (double)n16 * 16.0 * passes / (ms * 1e-3) / 1e9 : 0.0;
    return CUMF_OK;
}
