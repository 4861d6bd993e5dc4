// eval.cu - the evaluation criteria of LIBMF's mf-predict (test/mf-predict.cpp:21-35,
// test/mf.cpp:3794-4044) on the GPU.
//
// Pointwise criteria (MAE, GKL, LOGLOSS, ACCURACY) follow calc_rmse's layout: a group of 8
// lanes predicts one rating (mf_predict: float dot, b for ids outside the model or a NaN dot),
// lane 0 adds the term in double, blocks write partial sums and one thread adds them in order.
// The terms keep the reference's float / double mix (std:: float overloads of abs, log, exp,
// mf.cpp:3853, 3869, 3887-3889).
//
// Ranking criteria (row- / column-wise MPR and AUC, calc_mpr_auc mf.cpp:3913-4034).  For a
// row i with pos >= 1 positive test entries (r > 0) and n - pos >= 1 other columns, the
// reference moves the positives to the front of the row by swaps (mf.cpp:3995-3999), sorts
// them by prediction and, for every other column, counts the positives predicted strictly
// higher (u_auc) or not (u_mpr = pos (n - pos) - u_auc).  Here:
//   1. the test entries are sorted by (row, column) (CUB radix sort) and the positives kept;
//   2. one thread per row replays the swaps on column ids (the "positive block"; with no
//      repeated column it is the positive columns themselves);
//   3. the block's predictions are computed (sequential fp32 FMA over k, as
//      std::inner_product contracted to FMA) and sorted per row (CUB segmented sort);
//   4. a sweep CTA takes 16 rows: each thread predicts its columns for all 16 rows from the
//      transposed column factors (one global load feeds 16 FMAs) and counts, by binary search
//      in the sorted block predictions, the positives predicted higher;
//   5. the pairs inside the block are subtracted, and per-row terms are summed in row order.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/transform_iterator.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cumf_sgd.h"
#include "internal.h"
#include "train_common.h"

namespace cumf {

namespace {

enum { kRMSE = 0, kMAE = 1, kGKL = 2, kLOGLOSS = 5, kACC = 6, kRowMPR = 10, kColMPR = 11, kRowAUC = 12, kColAUC = 13 };

constexpr int kT = 256;
constexpr int kLanes = 8;
constexpr int kBlocks = 1024;
constexpr int kRowsPerSweep = 16;

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[kT / 32];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kT / 32; ++w) t += sh[w];
    return t;
}

template <int CRIT>
__global__ void __launch_bounds__(kT) pointwise_kernel(const cumf_node *__restrict__ R, uint64_t nnz,
                                                       const float *__restrict__ P, uint32_t m,
                                                       const float *__restrict__ Q, uint32_t n, int k, float b,
                                                       double *part) {
    const int lane = threadIdx.x % kLanes;
    const uint64_t group = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / kLanes;
    const uint64_t groups = (uint64_t)gridDim.x * blockDim.x / kLanes;
    const unsigned gmask = 0xffu << ((threadIdx.x & 31) & ~(kLanes - 1));
    double acc = 0.0;
    for (uint64_t i = group; i < nnz; i += groups) {
        const cumf_node x = R[i];
        const uint32_t u = (uint32_t)x.u, v = (uint32_t)x.v;
        float z = b;
        if (u < m && v < n) {
            const float *p = P + (uint64_t)u * k, *q = Q + (uint64_t)v * k;
            float s = 0.f;
            for (int c = lane; c < k; c += kLanes) s = __fmaf_rn(__ldg(p + c), __ldg(q + c), s);
            for (int o = kLanes / 2; o >= 1; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
            z = isnan(s) ? b : s;
        }
        if (lane == 0) {
            const float r = x.r;
            if (CRIT == kMAE) {
                acc += (double)fabsf(r - z);
            } else if (CRIT == kGKL) {
                acc += (double)(r * logf(r / z) - r + z);
            } else if (CRIT == kLOGLOSS) {
                acc += r > 0.f ? log(1.0 + (double)expf(-z)) : log(1.0 + (double)expf(z));
            } else {  // kACC
                acc += r > 0.f ? (z > 0.f ? 1.0 : 0.0) : (z < 0.f ? 1.0 : 0.0);
            }
        }
    }
    const double t = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void ordered_sum_kernel(const double *part, int64_t count, double *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0;
        for (int64_t i = 0; i < count; ++i) s += part[i];
        *out = s;
    }
}

// ---- ranking criteria ---------------------------------------------------------------------

// Keys (row << 32 | col) of the test entries, rows / columns swapped for the column-wise
// criteria; flags ids outside [0, rows) x [0, cols).
__global__ void keys_kernel(const cumf_node *__restrict__ R, int64_t nnz, int transpose, int32_t rows, int32_t cols,
                            uint64_t *keys, float *vals, int *bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const cumf_node x = R[i];
        const int32_t row = transpose ? x.v : x.u, col = transpose ? x.u : x.v;
        if (row < 0 || row >= rows || col < 0 || col >= cols) {
            atomicOr(bad, 1);
            keys[i] = 0;
        } else {
            keys[i] = ((uint64_t)(uint32_t)row << 32) | (uint32_t)col;
        }
        vals[i] = x.r;
    }
}

__device__ __forceinline__ int32_t key_row(uint64_t k) { return (int32_t)(k >> 32); }
__device__ __forceinline__ int32_t key_col(uint64_t k) { return (int32_t)(k & 0xffffffffu); }

// One thread per row segment of positives: the columns that end in positions [0, pos) after
// swap(row[q], row[index[q]]) for q = 0 .. pos-1 (mf.cpp:3995-3999), index ascending.
__global__ void block_kernel(const uint64_t *__restrict__ pkeys, const int64_t *__restrict__ seg_off, int64_t nseg,
                             int32_t *blk) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int64_t a = seg_off[s], pos = seg_off[s + 1] - a;
    bool dup = false;
    for (int64_t q = 1; q < pos && !dup; ++q) dup = key_col(pkeys[a + q]) == key_col(pkeys[a + q - 1]);
    if (!dup) {
        for (int64_t q = 0; q < pos; ++q) blk[a + q] = key_col(pkeys[a + q]);
        return;
    }
    // Positions below pos live in blk (identity until written); a position at or above pos is
    // only touched while it is the current target (targets never decrease).
    for (int64_t q = 0; q < pos; ++q) blk[a + q] = (int32_t)q;
    int64_t cur_key = -1;
    int32_t cur_val = 0;
    for (int64_t q = 0; q < pos; ++q) {
        const int64_t c = key_col(pkeys[a + q]);
        const int32_t x = blk[a + q];
        if (c < pos) {
            blk[a + q] = blk[a + c];
            blk[a + c] = x;
        } else {
            if (c != cur_key) {
                cur_key = c;
                cur_val = (int32_t)c;
            }
            blk[a + q] = cur_val;
            cur_val = x;
        }
    }
}

// mf_predict with a sequential fp32 FMA dot (std::inner_product, contracted).
__device__ __forceinline__ float seq_predict(const float *__restrict__ P, int32_t pm, const float *__restrict__ Q,
                                             int32_t qn, int k, float b, int32_t u, int32_t v) {
    if (u < 0 || u >= pm || v < 0 || v >= qn) return b;
    const float *p = P + (int64_t)u * k, *q = Q + (int64_t)v * k;
    float z = 0.f;
    for (int t = 0; t < k; ++t) z = __fmaf_rn(__ldg(p + t), __ldg(q + t), z);
    return isnan(z) ? b : z;
}

// Predictions of the block columns; row-major "row factors" R_f (rows x k) and "column
// factors" C_f (cols x k) already swapped for the column-wise criteria.
__global__ void block_pred_kernel(const uint64_t *__restrict__ pkeys, const int32_t *__restrict__ blk, int64_t total,
                                  const float *__restrict__ Rf, int32_t rf_rows, const float *__restrict__ Cf,
                                  int32_t cf_rows, int k, float b, float *pred) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < total; j += (int64_t)gridDim.x * blockDim.x)
        pred[j] = seq_predict(Rf, rf_rows, Cf, cf_rows, k, b, key_row(pkeys[j]), blk[j]);
}

// Number of entries of the ascending array s[0..len) greater than x.
__device__ __forceinline__ int64_t count_greater(const float *s, int64_t len, float x) {
    int64_t lo = 0, hi = len;  // first index with s[idx] > x
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (__ldg(s + mid) > x)
            hi = mid;
        else
            lo = mid + 1;
    }
    return len - lo;
}

// CTA over up to 16 active segments; threads stride over all columns [0, ncols_eff).
// CfT is the column factors transposed (k x cf_rows).
__global__ void __launch_bounds__(kT) sweep_kernel(const int64_t *__restrict__ active, int64_t nactive,
                                                   const int64_t *__restrict__ seg_off,
                                                   const int32_t *__restrict__ seg_row,
                                                   const float *__restrict__ sorted_pred,
                                                   const float *__restrict__ Rf, int32_t rf_rows,
                                                   const float *__restrict__ CfT, int32_t cf_rows,
                                                   int32_t ncols_eff, int k, float b,
                                                   unsigned long long *seg_count) {
    extern __shared__ float s_p[];  // kRowsPerSweep x k row factors
    __shared__ int64_t s_seg[kRowsPerSweep], s_off[kRowsPerSweep], s_len[kRowsPerSweep];
    __shared__ int s_valid[kRowsPerSweep];
    __shared__ unsigned long long s_cnt[kRowsPerSweep];
    const int64_t g0 = (int64_t)blockIdx.x * kRowsPerSweep;
    const int nr = (nactive - g0 < kRowsPerSweep) ? (int)(nactive - g0) : kRowsPerSweep;
    if (threadIdx.x < kRowsPerSweep) {
        const int r = threadIdx.x;
        s_cnt[r] = 0;
        if (r < nr) {
            const int64_t s = active[g0 + r];
            s_seg[r] = s;
            s_off[r] = seg_off[s];
            s_len[r] = seg_off[s + 1] - seg_off[s];
            s_valid[r] = seg_row[s] < rf_rows;
        } else {
            s_seg[r] = -1;
            s_off[r] = 0;
            s_len[r] = 0;
            s_valid[r] = 0;
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < kRowsPerSweep * k; idx += blockDim.x) {
        const int r = idx / k, t = idx % k;
        s_p[idx] = (r < nr && s_valid[r]) ? Rf[(int64_t)seg_row[s_seg[r]] * k + t] : 0.f;
    }
    __syncthreads();
    unsigned long long cnt[kRowsPerSweep];
#pragma unroll
    for (int r = 0; r < kRowsPerSweep; ++r) cnt[r] = 0;
    for (int32_t j = threadIdx.x; j < ncols_eff; j += blockDim.x) {
        float acc[kRowsPerSweep];
#pragma unroll
        for (int r = 0; r < kRowsPerSweep; ++r) acc[r] = 0.f;
        const bool in_model = j < cf_rows;
        if (in_model) {
            for (int t = 0; t < k; ++t) {
                const float q = __ldg(CfT + (int64_t)t * cf_rows + j);
#pragma unroll
                for (int r = 0; r < kRowsPerSweep; ++r) acc[r] = __fmaf_rn(s_p[r * k + t], q, acc[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < kRowsPerSweep; ++r) {
            if (r >= nr) continue;
            const float z = (in_model && s_valid[r] && !isnan(acc[r])) ? acc[r] : b;
            cnt[r] += (unsigned long long)count_greater(sorted_pred + s_off[r], s_len[r], z);
        }
    }
#pragma unroll
    for (int r = 0; r < kRowsPerSweep; ++r) {
        unsigned long long c = cnt[r];
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if ((threadIdx.x & 31) == 0 && r < nr) atomicAdd(&s_cnt[r], c);
    }
    __syncthreads();
    if (threadIdx.x < nr) seg_count[s_seg[threadIdx.x]] = s_cnt[threadIdx.x];
}

// Per segment: subtract the pairs inside the block, then this row's MPR and AUC terms.
__global__ void row_terms_kernel(const int64_t *__restrict__ seg_off, int64_t nseg, const float *__restrict__ sorted_pred,
                                 const unsigned long long *__restrict__ seg_count, int32_t ncols_eff, double *mpr,
                                 double *auc, int64_t *pos_out) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int64_t a = seg_off[s], pos = seg_off[s + 1] - a;
    if (ncols_eff - pos < 1 || pos < 1) {
        mpr[s] = 0;
        auc[s] = 0;
        pos_out[s] = 0;
        return;
    }
    unsigned long long within = 0;
    for (int64_t q = 0; q < pos; ++q) within += count_greater(sorted_pred + a, pos, sorted_pred[a + q]);
    const double u_auc = (double)(seg_count[s] - within);
    const double negs = (double)(ncols_eff - pos);
    mpr[s] = ((double)pos * negs - u_auc) / negs;
    auc[s] = u_auc / negs / (double)pos;
    pos_out[s] = pos;
}

// Row-order sums (the reference's serial order) of the per-row terms.
__global__ void finish_kernel(const double *mpr, const double *auc, const int64_t *pos, int64_t nseg, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double sm = 0, sa = 0;
    long long tm = 0, tp = 0;
    for (int64_t s = 0; s < nseg; ++s) {
        if (pos[s] == 0) continue;
        sm += mpr[s];
        sa += auc[s];
        tm += 1;
        tp += pos[s];
    }
    out[0] = sm / (double)tp;
    out[1] = sa / (double)tm;
}

__global__ void transpose_f32_kernel(const float *__restrict__ in, int64_t rows, int k, float *out) {
    // out[t * rows + i] = in[i * k + t]
    __shared__ float tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int t0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t i = i0 + y;
        const int t = t0 + threadIdx.x;
        tile[y][threadIdx.x] = (i < rows && t < k) ? in[i * k + t] : 0.f;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int t = t0 + y;
        const int64_t i = i0 + threadIdx.x;
        if (t < k && i < rows) out[(int64_t)t * rows + i] = tile[threadIdx.x][y];
    }
}

__global__ void seg_heads_kernel(const uint64_t *__restrict__ pkeys, int64_t total, const int64_t *__restrict__ head_pos,
                                 int64_t *seg_off, int32_t *seg_row) {
    // head_pos[j] = index of the segment starting at j (exclusive scan of head flags)
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < total; j += (int64_t)gridDim.x * blockDim.x) {
        if (j == 0 || key_row(pkeys[j]) != key_row(pkeys[j - 1])) {
            seg_off[head_pos[j]] = j;
            seg_row[head_pos[j]] = key_row(pkeys[j]);
        }
    }
}

struct HeadFlag {  // 1 where a row segment of the sorted positives starts (0 at j >= total)
    const uint64_t *keys;
    int64_t total;
    __device__ int64_t operator()(int64_t j) const {
        return (j < total && (j == 0 || key_row(keys[j]) != key_row(keys[j - 1]))) ? 1 : 0;
    }
};

struct PositiveFlag {
    const float *vals;
    __device__ char operator()(int64_t i) const { return vals[i] > 0.f ? 1 : 0; }
};

__global__ void active_kernel(const int64_t *__restrict__ seg_off, int64_t nseg, int32_t ncols_eff, int64_t *flag) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int64_t pos = seg_off[s + 1] - seg_off[s];
    flag[s] = (pos >= 1 && ncols_eff - pos >= 1) ? 1 : 0;
}

int grid_of(int64_t n, int per = kT) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, 65535 * 8)); }

// Device MPR and AUC (out[0], out[1]) for device records and float factors.
int mpr_auc_device(const cumf_node *d_R, int64_t nnz, int32_t prob_m, int32_t prob_n, const float *d_P, int32_t pm,
                   const float *d_Q, int32_t qn, int k, float b, int transpose, double *out, cudaStream_t s) {
    const int32_t rows = transpose ? std::max(prob_n, qn) : std::max(prob_m, pm);
    const int32_t cols = transpose ? std::max(prob_m, pm) : std::max(prob_n, qn);
    const float *Rf = transpose ? d_Q : d_P;
    const int32_t rf_rows = transpose ? qn : pm;
    const float *Cf = transpose ? d_P : d_Q;
    const int32_t cf_rows = transpose ? pm : qn;
    DevBuf keys, vals, skeys, svals, bad, idx, pidx, npos, tmp;
    CUMF_CUDA(keys.alloc(nnz * 8));
    CUMF_CUDA(vals.alloc(nnz * 4));
    CUMF_CUDA(skeys.alloc(nnz * 8));
    CUMF_CUDA(svals.alloc(nnz * 4));
    CUMF_CUDA(bad.alloc(sizeof(int)));
    CUMF_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    keys_kernel<<<grid_of(nnz), kT, 0, s>>>(d_R, nnz, transpose, rows, cols, keys.as<uint64_t>(), vals.as<float>(),
                                            bad.as<int>());
    CUMF_CUDA(cudaGetLastError());
    // 1. sort by (row, col); keep the positives.
    size_t tb = 0;
    CUMF_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys.as<uint64_t>(), skeys.as<uint64_t>(), vals.as<float>(),
                                              svals.as<float>(), nnz, 0, 64, s));
    CUMF_CUDA(tmp.alloc(tb));
    CUMF_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, keys.as<uint64_t>(), skeys.as<uint64_t>(), vals.as<float>(),
                                              svals.as<float>(), nnz, 0, 64, s));
    DevBuf pkeys, ntot;
    CUMF_CUDA(pkeys.alloc(nnz * 8));
    CUMF_CUDA(ntot.alloc(sizeof(int64_t)));
    {
        auto flags = thrust::make_transform_iterator(thrust::counting_iterator<int64_t>(0),
                                                     PositiveFlag{svals.as<float>()});
        size_t tb2 = 0;
        CUMF_CUDA(cub::DeviceSelect::Flagged(nullptr, tb2, skeys.as<uint64_t>(), flags, pkeys.as<uint64_t>(),
                                             ntot.as<int64_t>(), nnz, s));
        CUMF_CUDA(tmp.alloc(std::max(tb, tb2)));
        CUMF_CUDA(cub::DeviceSelect::Flagged(tmp.p, tb2, skeys.as<uint64_t>(), flags, pkeys.as<uint64_t>(),
                                             ntot.as<int64_t>(), nnz, s));
    }
    int64_t total = 0;
    int hbad = 0;
    CUMF_CUDA(cudaMemcpyAsync(&total, ntot.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    if (hbad) return fail(CUMF_ERR_RANGE, "evaluate: a test id is negative or outside the problem's extent");
    if (total == 0) {  // no row qualifies: 0 / 0 as in the reference
        out[0] = out[1] = NAN;
        return CUMF_OK;
    }
    // 2. row segments of the positives.
    DevBuf heads, seg_off, seg_row, nseg_d;
    CUMF_CUDA(heads.alloc((total + 1) * 8));
    {
        auto flags = thrust::make_transform_iterator(thrust::counting_iterator<int64_t>(0),
                                                     HeadFlag{pkeys.as<uint64_t>(), total});
        size_t tb3 = 0;
        CUMF_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb3, flags, heads.as<int64_t>(), total + 1, s));
        CUMF_CUDA(tmp.alloc(std::max<size_t>(tb3, 16)));
        CUMF_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb3, flags, heads.as<int64_t>(), total + 1, s));
    }
    // heads[total] = number of segments.
    int64_t nseg = 0;
    CUMF_CUDA(cudaMemcpyAsync(&nseg, heads.as<int64_t>() + total, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    CUMF_CUDA(seg_off.alloc((nseg + 1) * 8));
    CUMF_CUDA(seg_row.alloc(nseg * 4 + 4));
    seg_heads_kernel<<<grid_of(total), kT, 0, s>>>(pkeys.as<uint64_t>(), total, heads.as<int64_t>(),
                                                   seg_off.as<int64_t>(), seg_row.as<int32_t>());
    CUMF_CUDA(cudaMemcpyAsync(seg_off.as<int64_t>() + nseg, &total, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    // 3. positive blocks, their predictions, sorted per row.
    DevBuf blk, pred, spred;
    CUMF_CUDA(blk.alloc(total * 4));
    CUMF_CUDA(pred.alloc(total * 4));
    CUMF_CUDA(spred.alloc(total * 4));
    block_kernel<<<grid_of(nseg), kT, 0, s>>>(pkeys.as<uint64_t>(), seg_off.as<int64_t>(), nseg, blk.as<int32_t>());
    block_pred_kernel<<<grid_of(total), kT, 0, s>>>(pkeys.as<uint64_t>(), blk.as<int32_t>(), total, Rf, rf_rows, Cf,
                                                    cf_rows, k, b, pred.as<float>());
    CUMF_CUDA(cudaGetLastError());
    {
        size_t tb4 = 0;
        CUMF_CUDA(cub::DeviceSegmentedRadixSort::SortKeys(nullptr, tb4, pred.as<float>(), spred.as<float>(), total,
                                                          nseg, seg_off.as<int64_t>(), seg_off.as<int64_t>() + 1, 0,
                                                          32, s));
        CUMF_CUDA(tmp.alloc(std::max<size_t>(tb4, 16)));
        CUMF_CUDA(cub::DeviceSegmentedRadixSort::SortKeys(tmp.p, tb4, pred.as<float>(), spred.as<float>(), total,
                                                          nseg, seg_off.as<int64_t>(), seg_off.as<int64_t>() + 1, 0,
                                                          32, s));
    }
    // 4. active rows and the column sweep.
    DevBuf aflag, active, nact;
    CUMF_CUDA(aflag.alloc(nseg * 8));
    CUMF_CUDA(active.alloc(nseg * 8));
    CUMF_CUDA(nact.alloc(8));
    active_kernel<<<grid_of(nseg), kT, 0, s>>>(seg_off.as<int64_t>(), nseg, cols, aflag.as<int64_t>());
    {
        size_t tb5 = 0;
        CUMF_CUDA(cub::DeviceSelect::Flagged(nullptr, tb5, thrust::counting_iterator<int64_t>(0), aflag.as<int64_t>(),
                                             active.as<int64_t>(), nact.as<int64_t>(), nseg, s));
        CUMF_CUDA(tmp.alloc(std::max<size_t>(tb5, 16)));
        CUMF_CUDA(cub::DeviceSelect::Flagged(tmp.p, tb5, thrust::counting_iterator<int64_t>(0), aflag.as<int64_t>(),
                                             active.as<int64_t>(), nact.as<int64_t>(), nseg, s));
    }
    int64_t nactive = 0;
    CUMF_CUDA(cudaMemcpyAsync(&nactive, nact.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    DevBuf cfT, segcnt, mpr, auc, posb, res;
    CUMF_CUDA(segcnt.alloc(nseg * 8));
    CUMF_CUDA(cudaMemsetAsync(segcnt.p, 0, nseg * 8, s));
    if (nactive > 0) {
        CUMF_CUDA(cfT.alloc((size_t)cf_rows * k * 4));
        if (cf_rows > 0) {
            dim3 tg((unsigned)((cf_rows + 31) / 32), (unsigned)((k + 31) / 32));
            transpose_f32_kernel<<<tg, dim3(32, 8), 0, s>>>(Cf, cf_rows, k, cfT.as<float>());
        }
        const size_t smem = (size_t)kRowsPerSweep * k * sizeof(float);
        if (smem > 48 * 1024)
            CUMF_CUDA(cudaFuncSetAttribute(sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int64_t groups = (nactive + kRowsPerSweep - 1) / kRowsPerSweep;
        if (groups > 0x7fffffffll) return fail(CUMF_ERR_ARG, "evaluate: too many rows");
        sweep_kernel<<<(unsigned)groups, kT, smem, s>>>(active.as<int64_t>(), nactive, seg_off.as<int64_t>(),
                                                        seg_row.as<int32_t>(), spred.as<float>(), Rf, rf_rows,
                                                        cfT.as<float>(), cf_rows, cols, k, b,
                                                        segcnt.as<unsigned long long>());
        CUMF_CUDA(cudaGetLastError());
    }
    // 5. row terms, summed in row order.
    CUMF_CUDA(mpr.alloc(nseg * 8));
    CUMF_CUDA(auc.alloc(nseg * 8));
    CUMF_CUDA(posb.alloc(nseg * 8));
    CUMF_CUDA(res.alloc(16));
    row_terms_kernel<<<grid_of(nseg), kT, 0, s>>>(seg_off.as<int64_t>(), nseg, spred.as<float>(),
                                                  segcnt.as<unsigned long long>(), cols, mpr.as<double>(),
                                                  auc.as<double>(), posb.as<int64_t>());
    finish_kernel<<<1, 32, 0, s>>>(mpr.as<double>(), auc.as<double>(), posb.as<int64_t>(), nseg, res.as<double>());
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(cudaMemcpyAsync(out, res.p, 16, cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    return CUMF_OK;
}

}  // namespace

}  // namespace cumf

using namespace cumf;

extern "C" int cumf_evaluate(const cumf_problem *te, const cumf_model *model, int criterion, double *out) {
    TraceRange trace("evaluate (mf-predict criterion)");
    if (!te || !model || !out) return fail(CUMF_ERR_ARG, "evaluate: NULL argument");
    const bool ranking = criterion >= kRowMPR && criterion <= kColAUC;
    if (!(criterion == kRMSE || criterion == kMAE || criterion == kGKL || criterion == kLOGLOSS || criterion == kACC ||
          ranking))
        return fail(CUMF_ERR_ARG, "unknown evaluation criterion");
    if (criterion == kRMSE) return cumf_rmse(te, model, out);
    if (te->nnz == 0 && !ranking) {  // the pointwise criteria return 0 for an empty set
        *out = 0;
        return CUMF_OK;
    }
    if ((te->nnz > 0 && !te->R) || (!model->P && model->m > 0) || (!model->Q && model->n > 0) || model->k <= 0)
        return fail(CUMF_ERR_ARG, "evaluate: malformed input");
    if (int rc = select_device(0)) return rc;
    Stream stream;
    CUMF_CUDA(cudaStreamCreateWithFlags(&stream.s, cudaStreamNonBlocking));
    DevBuf d_R, d_P, d_Q, d_part, d_sum;
    const size_t pb = (size_t)model->m * model->k * sizeof(float), qb = (size_t)model->n * model->k * sizeof(float);
    CUMF_CUDA(d_R.alloc(std::max<int64_t>(1, te->nnz) * sizeof(cumf_node)));
    CUMF_CUDA(d_P.alloc(pb));
    CUMF_CUDA(d_Q.alloc(qb));
    if (te->nnz)
        CUMF_CUDA(cudaMemcpyAsync(d_R.p, te->R, te->nnz * sizeof(cumf_node), cudaMemcpyHostToDevice, stream.s));
    if (pb) CUMF_CUDA(cudaMemcpyAsync(d_P.p, model->P, pb, cudaMemcpyHostToDevice, stream.s));
    if (qb) CUMF_CUDA(cudaMemcpyAsync(d_Q.p, model->Q, qb, cudaMemcpyHostToDevice, stream.s));
    if (ranking) {
        if (te->nnz == 0) {
            *out = NAN;  // 0 / 0 (mf.cpp:4029-4030)
            return CUMF_OK;
        }
        double two[2] = {0, 0};
        const int transpose = (criterion == kColMPR || criterion == kColAUC);
        if (int rc = mpr_auc_device(d_R.as<cumf_node>(), te->nnz, te->m, te->n, d_P.as<float>(), model->m,
                                    d_Q.as<float>(), model->n, model->k, model->b, transpose, two, stream.s))
            return rc;
        *out = (criterion == kRowMPR || criterion == kColMPR) ? two[0] : two[1];
        return CUMF_OK;
    }
    CUMF_CUDA(d_part.alloc(kBlocks * sizeof(double)));
    CUMF_CUDA(d_sum.alloc(sizeof(double)));
    const cumf_node *R = d_R.as<cumf_node>();
    const uint64_t nnz = (uint64_t)te->nnz;
    const float *P = d_P.as<float>(), *Q = d_Q.as<float>();
    const uint32_t m = (uint32_t)model->m, n = (uint32_t)model->n;
    switch (criterion) {
        case kMAE: pointwise_kernel<kMAE><<<kBlocks, kT, 0, stream.s>>>(R, nnz, P, m, Q, n, model->k, model->b, d_part.as<double>()); break;
        case kGKL: pointwise_kernel<kGKL><<<kBlocks, kT, 0, stream.s>>>(R, nnz, P, m, Q, n, model->k, model->b, d_part.as<double>()); break;
        case kLOGLOSS: pointwise_kernel<kLOGLOSS><<<kBlocks, kT, 0, stream.s>>>(R, nnz, P, m, Q, n, model->k, model->b, d_part.as<double>()); break;
        default: pointwise_kernel<kACC><<<kBlocks, kT, 0, stream.s>>>(R, nnz, P, m, Q, n, model->k, model->b, d_part.as<double>()); break;
    }
    ordered_sum_kernel<<<1, 32, 0, stream.s>>>(d_part.as<double>(), kBlocks, d_sum.as<double>());
    CUMF_CUDA(cudaGetLastError());
    double sum = 0;
    CUMF_CUDA(cudaMemcpyAsync(&sum, d_sum.p, sizeof(double), cudaMemcpyDeviceToHost, stream.s));
    CUMF_CUDA(cudaStreamSynchronize(stream.s));
    *out = sum / (double)te->nnz;
    return CUMF_OK;
}
