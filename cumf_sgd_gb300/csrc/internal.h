// internal.h - declarations shared by the library's translation units (not exported).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "cumf_sgd.h"

namespace cumf {

// ---- tracing ---------------------------------------------------------------------------
// An NVTX range around a pipeline stage (prep, epochs, export, evaluation, ...), visible in
// Nsight Systems / Nsight Compute timelines; without a tool attached a push/pop is a no-op
// call.  end() closes the range early; the destructor closes it on every return path.
class TraceRange {
  public:
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { end(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
    void end() {
        if (open_) nvtxRangePop();
        open_ = false;
    }

  private:
    bool open_ = true;
};

// ---- error reporting ---------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define CUMF_CUDA(call)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// ---- schedule helpers ----------------------------------------------------------------
inline int64_t batches_per_worker(int64_t nnz, int workers) {
    // ceil(nnz / (workers * 128)) as in sgd_kernel.cu:203 (computed in integers).
    const int64_t per = (int64_t)workers * 128;
    return (nnz + per - 1) / per;
}

// ---- sgd_update.cu -------------------------------------------------------------------
struct Tuning {
    int lanes = 0;      // 0 = default
    int prefetch = -1;  // -1 = default
    int hints = -1;     // -1 = default
    int ring = -1;      // -1 = default, 0 = register prefetch kernel, 1 = shared-memory ring kernel
    int freeze_q = 0;   // 1 = item rows are not written
    int copies = 0;     // 1 = the ratings name copies of hot rows (default prefetch follows)
};
Tuning resolve_tuning(int k, int precision, Tuning t);
int default_lanes(int k, int precision);
bool lanes_supported(int k, int precision, int lanes);
int workers_per_block(int lanes);
int resident_workers(int k, int precision, int lanes, int sm_count);
cudaError_t launch_sgd_update(const cumf_node *d_R, int64_t nnz, void *d_P, int32_t m,
                              void *d_Q, int32_t n, int k, int precision, int num_workers,
                              const Tuning &tuning, const float *d_lr, int first_epoch,
                              int n_epochs, float lambda_p, float lambda_q, uint64_t seed,
                              int *d_status, cudaStream_t stream, int *lanes_used);

// ---- prep.cu ---------------------------------------------------------------------------
// index_offset: element index of d[0] in the whole matrix (segments of modes B/C draw the
// same values as the whole matrix would).
cudaError_t launch_init_factors(void *d, int64_t rows, int k, int precision, uint64_t seed,
                                uint32_t tag, cudaStream_t s, uint64_t index_offset = 0);
// Seed of the sample stream of grid block g (block 0 keeps the run's seed).
inline uint64_t block_seed(uint64_t seed, int g) { return seed + (uint64_t)g * 0x9E3779B97F4A7C15ull; }
// Partial sums (sum r, sum r^2) per block into d_part[2*blocks]; returns blocks used.
int stats_blocks(int64_t nnz);
cudaError_t launch_rating_stats(const cumf_node *d_R, int64_t nnz, double *d_part,
                                double *d_out2, cudaStream_t s);
cudaError_t launch_shuffle_scale(const cumf_node *in, cumf_node *out, int64_t nnz,
                                 const int32_t *pmap, int32_t m, const int32_t *qmap,
                                 int32_t n, float scale, int *d_status, cudaStream_t s);
cudaError_t launch_export(const void *in, int precision, const int32_t *map, int64_t rows,
                          int k, float factor, float *out, cudaStream_t s);
// dst[map[o]] = storage(src[o] / factor): starting factors in storage layout.
cudaError_t launch_import(const float *src, const int32_t *map, int64_t rows, int k, float factor, void *dst,
                          int precision, cudaStream_t s);
int rmse_blocks(int64_t nnz);
cudaError_t launch_rmse(const cumf_node *d_R, int64_t nnz, const float *P, int32_t m,
                        const float *Q, int32_t n, int k, float b, double *d_part,
                        double *d_sum, cudaStream_t s);
// The same evaluator on a caller-chosen grid: d_part holds `blocks` partials.
cudaError_t launch_rmse_grid(const cumf_node *d_R, int64_t nnz, const float *P, int32_t m,
                             const float *Q, int32_t n, int k, float b, int blocks,
                             double *d_part, double *d_sum, cudaStream_t s);
// Loads launch_rmse_grid's kernels onto the current device without launching them.
cudaError_t load_rmse_kernels();

// Order-independent digest of `bytes` (a multiple of 4) at d into *d_out.
cudaError_t launch_digest(const void *d, uint64_t bytes, unsigned long long *d_out, cudaStream_t s);

// f(a, b, t) over [0, n) split into contiguous chunks, one per host thread (at most 16).
template <typename F>
void parallel_chunks(int64_t n, F f) {
    const int64_t T = std::max<int64_t>(1, std::min<int64_t>(std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency())),
                                                             n / 65536 + 1));
    std::vector<std::thread> th;
    for (int64_t t = 0; t < T; ++t) th.emplace_back([&, t] { f(n * t / T, n * (t + 1) / T, (int)t); });
    for (auto &x : th) x.join();
}

// grid_problem's in-place bucketing (sgd.cu:455-482) replayed on block ids: fin[slot] = the
// original index of the record that the reference's cycle swaps leave in that slot.  bid[i]
// is record i's block (0 <= bid < G); grid_size holds the counts.  Same order as swapping the
// records, without moving them: each step reads one block id and writes one index.
void grid_order(const int32_t *bid, int64_t nnz, int G, const int64_t *grid_size, int64_t *fin);

// ---- strata.cu (deterministic training) ---------------------------------------------------
// The strata of epoch ep in their seeded random order (a permutation of 0 .. G-1).
void strata_order(uint64_t seed, int ep, int G, int *order);
// Groups per side of the stratified grid: `requested` when > 1, else about sqrt(nnz / 24).
int strata_groups(int64_t nnz, int requested);
// d_out: the ratings stably sorted by block (u mod G) * G + (v mod G); d_block_off: G*G + 1
// block offsets.  Synchronises the stream.
int strata_layout(const cumf_node *d_R, int64_t nnz, int G, cumf_node *d_out, unsigned long long *d_block_off,
                  cudaStream_t s);
// Epochs [first_epoch, first_epoch + n_epochs): G strata each, learning rates h_lr[epoch] (host).
int strata_epochs(const cumf_node *d_S, const unsigned long long *d_block_off, int G, void *d_P, int32_t m,
                  void *d_Q, int32_t n, int k, int precision, const float *h_lr, int first_epoch, int n_epochs,
                  float lambda_p, float lambda_q, uint64_t seed, int *d_status, cudaStream_t s);

// ---- hot_rows.cu (copies of the most-rated rows) ----------------------------------------
// A copy carries at least this many ratings an epoch, and a row has at most kHotMaxCopies.
constexpr int64_t kHotMinPerCopy = 4096;
constexpr int kHotMaxCopies = 256;
// cumf_params.hot_rows of cumf_default_params: 0, no copies (every rating updates its own
// rows, as the reference's kernel).  0.5 is the measured setting for skewed item popularity
// (480,189 x 17,770: 12.6 -> 8.7 ms per epoch at a lower test RMSE); it is not the default
// because on 1,000,990 x 624,961 with rating noise as large as the signal the copies raised
// the test RMSE after 20 epochs (fp16 30.76 -> 31.51, fp32 30.33 -> 30.81).
constexpr float kHotDefaultConcurrency = 0.0f;
// Ratings per copy for `concurrency` expected workers on one copy at a time (0 = no copies:
// concurrency <= 0, fewer than two workers or no ratings).
int64_t hot_rows_per_copy(int64_t nnz, int32_t num_workers, int k, int precision, int lanes, float concurrency,
                          int sm_count);
// Rows of a plan before (m, n) and with (m_rows, n_rows) the copies.
void hot_rows_dims(const cumf_hot_rows *h, int32_t *m, int32_t *n, int32_t *m_rows, int32_t *n_rows);
// Size in bytes of one factor element for a precision.
inline int elem_bytes(int precision) { return precision == CUMF_FP32 ? 4 : 2; }

}  // namespace cumf
