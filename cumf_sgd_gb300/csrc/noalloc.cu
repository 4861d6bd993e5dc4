// noalloc.cu - an RMSE entry point that allocates no memory.
//
// cumf_dev_rmse gets its per-block partial sums from cudaMalloc.  Some callers cannot
// allocate device memory at the point where they want an evaluation: code running inside a
// memory pool or arena that must not grow, allocator hooks and out-of-memory handlers, and
// callers that hand this library only fixed, pre-sized buffers.  For them,
// cumf_dev_rmse_noalloc keeps its scratch in a file-scope __device__ array of fixed size that
// every GPU loading the library holds until the process exits.
//
// Limits and behaviour:
//  - the scratch holds kNoAllocMaxBlocks partial sums plus one total; the evaluator uses one
//    block per kNoAllocRatingsPerBlock ratings, so at most
//    kNoAllocMaxBlocks * kNoAllocRatingsPerBlock (134,217,728) ratings per call; larger
//    calls fail with CUMF_ERR_ARG before anything is launched;
//  - every scratch slot a call reads is written earlier in the same call (each block writes
//    its partial, the final pass writes the total), so nothing needs clearing between calls;
//  - all calls share the one array: calls whose kernels overlap on the GPU (different
//    streams, or different host threads) race on it and must be serialised by the caller;
//  - the first call on a device, with that device current, is its set-up: it looks up the
//    array's device address (cudaGetSymbolAddress), caches it, and loads the evaluator
//    kernels.  Under CUDA's lazy module loading (the default) loading device code allocates,
//    so that first call must come where allocation is still possible (at start-up, say) and
//    before any stream capture; a call with nnz = 0 does the set-up and nothing else;
//  - the cached address belongs to the device's current context: after a cudaDeviceReset
//    in the same process it is stale, so the entry point must not be used across a reset;
//  - the result equals cumf_dev_rmse's within the rounding of the double sum (the two split
//    the ratings into different blocks) and is the same bits from call to call.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>
#include <string>

#include "cumf_sgd.h"
#include "internal.h"

namespace cumf {

namespace {

constexpr int kNoAllocMaxBlocks = 16384;
constexpr int64_t kNoAllocRatingsPerBlock = 8192;

// [0, kNoAllocMaxBlocks): per-block partial sums; [kNoAllocMaxBlocks]: the total.
static __device__ __align__(256) double g_rmse_scratch[kNoAllocMaxBlocks + 1];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (looked up once per device).
int scratch_for_current_device(double **out) {
    int dev = 0;
    CUMF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(CUMF_ERR_ARG, "device index out of range for the no-alloc scratch");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rmse_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_rmse_scratch)");
        e = load_rmse_kernels();
        if (e != cudaSuccess) return cuda_fail(e, "loading the evaluator kernels");
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return CUMF_OK;
}

}  // namespace

}  // namespace cumf

using namespace cumf;

extern "C" int cumf_dev_rmse_noalloc(const cumf_node *d_R, int64_t nnz, const float *d_P, int32_t m,
                                     const float *d_Q, int32_t n, int k, float b, double *out_rmse,
                                     void *stream) {
    if (nnz < 0 || k <= 0 || !out_rmse || (nnz > 0 && (!d_R || !d_P || !d_Q)))
        return fail(CUMF_ERR_ARG, "dev_rmse_noalloc: bad arguments");
    const int64_t max_nnz = (int64_t)kNoAllocMaxBlocks * kNoAllocRatingsPerBlock;
    if (nnz > max_nnz)
        return fail(CUMF_ERR_ARG, "dev_rmse_noalloc: " + std::to_string(nnz) +
                                      " ratings exceed the fixed scratch limit of " + std::to_string(max_nnz));
    double *scratch = nullptr;
    if (int rc = scratch_for_current_device(&scratch)) return rc;
    if (nnz == 0) {  // set-up only
        *out_rmse = 0;
        return CUMF_OK;
    }
    const int blocks = (int)((nnz + kNoAllocRatingsPerBlock - 1) / kNoAllocRatingsPerBlock);
    cudaStream_t s = (cudaStream_t)stream;
    CUMF_CUDA(launch_rmse_grid(d_R, nnz, d_P, m, d_Q, n, k, b, blocks, scratch, scratch + kNoAllocMaxBlocks, s));
    double sum = 0;
    CUMF_CUDA(cudaMemcpyAsync(&sum, scratch + kNoAllocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    *out_rmse = sqrt(sum / (double)nnz);
    return CUMF_OK;
}
