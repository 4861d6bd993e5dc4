// hot_rows.cu - copies of the most-rated user and item rows for batch-Hogwild epochs.
//
// No counterpart in the reference: its update kernel (sgd_k128_kernel_hogwild_warp32.h:3-104)
// reads and writes one row of P and one row of Q per rating, whatever the ids.  With skewed
// ids many resident workers hold the same row at the same moment, and the lines of those rows
// serialise the whole epoch: at 480,189 x 17,770 with 99M ratings (Zipf item popularity, the
// most-rated item has about 230,000 ratings, 40x the mean) an epoch takes 13.0 ms on GB300;
// the same ratings with uniformly drawn item ids take 9.8 ms, wherever the rows are placed.
//
// A row with more than `per_copy` ratings gets copies = min(max_copies, ceil(count / per_copy))
// copies: the row itself and copies - 1 extra rows appended after the last row of its matrix
// (in row order, so the layout is a function of the counts alone).  Rating i of such a row
// is assigned copy i mod copies, and the ratings are rewritten once to name their copy.  The
// copies start equal (spread) and are averaged after every launch of epochs (merge): the mean
// of the copies in fp32, summed in copy order, rounded to nearest in the storage type and
// written to every copy.  Each copy sees 1/copies of its row's ratings, so the workers that
// would have queued on one row spread over several; the average then stands for the row.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "device_common.cuh"
#include "internal.h"
#include "train_common.h"

struct cumf_hot_rows {
    int32_t m = 0, n = 0;            // rows of P and Q before the copies
    int32_t m_rows = 0, n_rows = 0;  // rows including the copies
    int32_t hot_m = 0, hot_n = 0;    // rows that have copies
    int64_t per_copy = 0;
    int32_t max_copies = 0;
    int device = 0;
    cumf::DevBuf mem;
    int2 *tab_m = nullptr, *tab_n = nullptr;      // per row: {copies, first extra row}
    int32_t *grp_m = nullptr, *grp_n = nullptr;   // the rows with copies, ascending
};

namespace cumf {
namespace {

constexpr int kThreads = 256;
constexpr int kPlanThreads = 1024;

int count_grid(uint64_t items) {
    uint64_t b = (items + kThreads * 4ull - 1) / (kThreads * 4ull);
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(b, 152ull * 16));
}

__global__ void hot_count_kernel(const cumf_node *R, uint64_t nnz, uint32_t m, uint32_t n,
                                 unsigned long long *cnt_m, unsigned long long *cnt_n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nnz;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t u = (uint32_t)R[i].u, v = (uint32_t)R[i].v;
        if (u < m) atomicAdd(&cnt_m[u], 1ull);
        if (v < n) atomicAdd(&cnt_n[v], 1ull);
    }
}

__device__ __forceinline__ int copies_of(unsigned long long c, unsigned long long per_copy, int max_copies) {
    if (c <= per_copy) return 1;
    const unsigned long long q = (c + per_copy - 1) / per_copy;
    return q >= (unsigned long long)max_copies ? max_copies : (int)q;
}

// Exclusive scan of (a, b) over the block; returns the block totals in *ta, *tb.
__device__ void block_scan2(long long &a, long long &b, long long *ta, long long *tb) {
    __shared__ long long wa[kPlanThreads / 32], wb[kPlanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long ia = a, ib = b;  // inclusive within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const long long xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
            ia += xa;
            ib += xb;
        }
    }
    if (lane == 31) {
        wa[w] = ia;
        wb[w] = ib;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long sa = 0, sb = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            const long long xa = wa[i], xb = wb[i];
            wa[i] = sa;
            wb[i] = sb;
            sa += xa;
            sb += xb;
        }
        *ta = sa;
        *tb = sb;
    }
    __syncthreads();
    a = wa[w] + ia - a;
    b = wb[w] + ib - b;
}

// One block per matrix (block 0: users, block 1: items).  Each thread owns a contiguous run
// of rows; the runs' (extra rows, rows with copies) are scanned across the block, then every
// row's entry and the list of rows with copies are written in row order.
__global__ void __launch_bounds__(kPlanThreads) hot_plan_kernel(
    const unsigned long long *cnt_m, int32_t m, const unsigned long long *cnt_n, int32_t n,
    unsigned long long per_copy, int max_copies, int2 *tab_m, int2 *tab_n, int32_t *grp_m, int32_t *grp_n,
    long long *totals) {
    const bool items = blockIdx.x == 1;
    const unsigned long long *cnt = items ? cnt_n : cnt_m;
    const int64_t rows = items ? n : m;
    int2 *tab = items ? tab_n : tab_m;
    int32_t *grp = items ? grp_n : grp_m;
    const int64_t chunk = (rows + blockDim.x - 1) / blockDim.x;
    const int64_t lo = std::min<int64_t>(rows, (int64_t)threadIdx.x * chunk), hi = std::min<int64_t>(rows, lo + chunk);
    long long extra = 0, hot = 0;
    for (int64_t r = lo; r < hi; ++r) {
        const int c = copies_of(cnt[r], per_copy, max_copies);
        extra += c - 1;
        hot += c > 1;
    }
    __shared__ long long tot[2];
    block_scan2(extra, hot, &tot[0], &tot[1]);
    for (int64_t r = lo; r < hi; ++r) {
        const int c = copies_of(cnt[r], per_copy, max_copies);
        tab[r] = make_int2(c, c > 1 ? (int)(rows + extra) : (int)r);
        if (c > 1) {
            grp[hot++] = (int32_t)r;
            extra += c - 1;
        }
    }
    if (threadIdx.x == 0) {
        totals[2 * blockIdx.x] = tot[0];
        totals[2 * blockIdx.x + 1] = tot[1];
    }
}

__global__ void hot_assign_kernel(cumf_node *R, uint64_t nnz, const int2 *tab_m, uint32_t m, const int2 *tab_n,
                                  uint32_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nnz;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (tab_m) {
            const uint32_t u = (uint32_t)R[i].u;
            if (u < m) {
                const int2 t = tab_m[u];
                if (t.x > 1) {
                    const int r = (int)(i % (uint64_t)t.x);
                    if (r) R[i].u = t.y + r - 1;
                }
            }
        }
        if (tab_n) {
            const uint32_t v = (uint32_t)R[i].v;
            if (v < n) {
                const int2 t = tab_n[v];
                if (t.x > 1) {
                    const int r = (int)(i % (uint64_t)t.x);
                    if (r) R[i].v = t.y + r - 1;
                }
            }
        }
    }
}

// One block per row with copies (users first, then items), one thread per element.
// merge = 0: every extra row takes the row's bits.  merge = 1: every copy takes the rounded
// mean of all copies.
template <int KIND>
__global__ void hot_merge_kernel(void *P, const int2 *tab_m, const int32_t *grp_m, int hot_m, void *Q,
                                 const int2 *tab_n, const int32_t *grp_n, int k, int merge) {
    using S = Scalar<KIND>;
    using T = typename S::T;
    int g = blockIdx.x;
    T *F = static_cast<T *>(P);
    const int2 *tab = tab_m;
    const int32_t *grp = grp_m;
    if (g >= hot_m) {
        g -= hot_m;
        F = static_cast<T *>(Q);
        tab = tab_n;
        grp = grp_n;
    }
    const int64_t row = grp[g];
    const int2 t = tab[row];
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        T *own = F + row * k + j;
        T out = *own;
        if (merge) {
            float acc = S::to_float(out);
            for (int c = 0; c < t.x - 1; ++c) acc += S::to_float(F[((int64_t)t.y + c) * k + j]);
            out = S::from_float(acc / (float)t.x);
            *own = out;
        }
        for (int c = 0; c < t.x - 1; ++c) F[((int64_t)t.y + c) * k + j] = out;
    }
}

int merge_launch(const cumf_hot_rows *h, void *d_P, void *d_Q, int k, int precision, int merge, cudaStream_t s) {
    const int blocks = h->hot_m + h->hot_n;
    if (blocks == 0) return CUMF_OK;
    if ((h->hot_m && !d_P) || (h->hot_n && !d_Q)) return fail(CUMF_ERR_ARG, "hot rows: NULL factor matrix");
    const int threads = std::min(k, 256);
    switch (store_of_precision(precision)) {
        case kHalf:
            hot_merge_kernel<kHalf><<<blocks, threads, 0, s>>>(d_P, h->tab_m, h->grp_m, h->hot_m, d_Q, h->tab_n,
                                                               h->grp_n, k, merge);
            break;
        case kBf16:
            hot_merge_kernel<kBf16><<<blocks, threads, 0, s>>>(d_P, h->tab_m, h->grp_m, h->hot_m, d_Q, h->tab_n,
                                                               h->grp_n, k, merge);
            break;
        default:
            hot_merge_kernel<kFloat><<<blocks, threads, 0, s>>>(d_P, h->tab_m, h->grp_m, h->hot_m, d_Q, h->tab_n,
                                                                h->grp_n, k, merge);
            break;
    }
    CUMF_CUDA(cudaGetLastError());
    return CUMF_OK;
}

}  // namespace

int64_t hot_rows_per_copy(int64_t nnz, int32_t num_workers, int k, int precision, int lanes, float concurrency,
                          int sm_count) {
    if (!(concurrency > 0.f) || nnz <= 0 || num_workers < 2) return 0;
    const int l = lanes > 0 ? lanes : default_lanes(k, precision);
    const int64_t resident = std::max(1, resident_workers(k, precision, l, sm_count));
    const int64_t w = std::min<int64_t>(num_workers, resident);
    // Expected workers on one row at a time = w * count / nnz; a copy carries at most
    // `concurrency` of them, and never fewer than kHotMinPerCopy ratings an epoch.
    const double t = std::ceil((double)nnz * (double)concurrency / (double)w);
    return std::max<int64_t>(kHotMinPerCopy, (int64_t)std::min(t, 9.0e18));
}

void hot_rows_dims(const cumf_hot_rows *h, int32_t *m, int32_t *n, int32_t *m_rows, int32_t *n_rows) {
    *m = h->m;
    *n = h->n;
    *m_rows = h->m_rows;
    *n_rows = h->n_rows;
}

}  // namespace cumf

using namespace cumf;

extern "C" {

int64_t cumf_hot_rows_per_copy(int64_t nnz, int32_t num_workers, int k, int precision, int lanes,
                               float concurrency) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    return hot_rows_per_copy(nnz, num_workers, k, precision, lanes, concurrency, sms);
}

int cumf_hot_rows_plan(const cumf_node *d_R, int64_t nnz, int32_t m, int32_t n, int64_t per_copy,
                       int32_t max_copies, cumf_hot_rows **out, void *stream) {
    TraceRange trace("hot rows: plan");
    if (!out) return fail(CUMF_ERR_ARG, "hot_rows_plan: NULL output");
    *out = nullptr;
    if (nnz < 0 || m < 1 || n < 1 || per_copy < 1 || max_copies < 1 || (nnz > 0 && !d_R))
        return fail(CUMF_ERR_ARG, "hot_rows_plan: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    cumf_hot_rows *h = new cumf_hot_rows();
    h->m = h->m_rows = m;
    h->n = h->n_rows = n;
    h->per_copy = per_copy;
    h->max_copies = max_copies;
    cudaGetDevice(&h->device);
    auto bail = [&](int rc) {
        delete h;
        return rc;
    };
    // tab_m | tab_n | grp_m | grp_n, each 16-byte aligned.
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t b_tm = up16((size_t)m * sizeof(int2)), b_tn = up16((size_t)n * sizeof(int2));
    const size_t b_gm = up16((size_t)m * sizeof(int32_t)), b_gn = up16((size_t)n * sizeof(int32_t));
    cudaError_t e = h->mem.alloc(b_tm + b_tn + b_gm + b_gn);
    if (e != cudaSuccess) return bail(cuda_fail(e, "hot_rows_plan: tables"));
    char *base = h->mem.as<char>();
    h->tab_m = reinterpret_cast<int2 *>(base);
    h->tab_n = reinterpret_cast<int2 *>(base + b_tm);
    h->grp_m = reinterpret_cast<int32_t *>(base + b_tm + b_tn);
    h->grp_n = reinterpret_cast<int32_t *>(base + b_tm + b_tn + b_gm);
    DevBuf cnt;
    e = cnt.alloc(((size_t)m + n) * sizeof(unsigned long long) + 4 * sizeof(long long));
    if (e != cudaSuccess) return bail(cuda_fail(e, "hot_rows_plan: counts"));
    unsigned long long *cnt_m = cnt.as<unsigned long long>(), *cnt_n = cnt_m + m;
    long long *d_tot = reinterpret_cast<long long *>(cnt_n + n);
    e = cudaMemsetAsync(cnt.p, 0, cnt.bytes, s);
    if (e == cudaSuccess && nnz > 0) {
        hot_count_kernel<<<count_grid((uint64_t)nnz), kThreads, 0, s>>>(d_R, (uint64_t)nnz, (uint32_t)m, (uint32_t)n,
                                                                         cnt_m, cnt_n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        hot_plan_kernel<<<2, kPlanThreads, 0, s>>>(cnt_m, m, cnt_n, n, (unsigned long long)per_copy, max_copies,
                                                   h->tab_m, h->tab_n, h->grp_m, h->grp_n, d_tot);
        e = cudaGetLastError();
    }
    long long tot[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(tot, d_tot, sizeof(tot), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return bail(cuda_fail(e, "hot_rows_plan"));
    if ((long long)m + tot[0] > 0x7fffffffll || (long long)n + tot[2] > 0x7fffffffll)
        return bail(fail(CUMF_ERR_ARG, "hot_rows_plan: more than 2^31 - 1 rows with the copies"));
    h->m_rows = (int32_t)(m + tot[0]);
    h->hot_m = (int32_t)tot[1];
    h->n_rows = (int32_t)(n + tot[2]);
    h->hot_n = (int32_t)tot[3];
    *out = h;
    return CUMF_OK;
}

int cumf_hot_rows_info(const cumf_hot_rows *h, int32_t *m_rows, int32_t *n_rows, int32_t *hot_m, int32_t *hot_n) {
    if (!h) return fail(CUMF_ERR_ARG, "hot_rows_info: NULL plan");
    if (m_rows) *m_rows = h->m_rows;
    if (n_rows) *n_rows = h->n_rows;
    if (hot_m) *hot_m = h->hot_m;
    if (hot_n) *hot_n = h->hot_n;
    return CUMF_OK;
}

int cumf_hot_rows_tables(const cumf_hot_rows *h, int32_t *tab_m, int32_t *tab_n, int32_t *grp_m, int32_t *grp_n) {
    if (!h) return fail(CUMF_ERR_ARG, "hot_rows_tables: NULL plan");
    const struct {
        void *dst;
        const void *src;
        size_t bytes;
    } parts[4] = {{tab_m, h->tab_m, (size_t)h->m * sizeof(int2)},
                  {tab_n, h->tab_n, (size_t)h->n * sizeof(int2)},
                  {grp_m, h->grp_m, (size_t)h->hot_m * sizeof(int32_t)},
                  {grp_n, h->grp_n, (size_t)h->hot_n * sizeof(int32_t)}};
    for (const auto &x : parts)
        if (x.dst && x.bytes) CUMF_CUDA(cudaMemcpy(x.dst, x.src, x.bytes, cudaMemcpyDefault));
    return CUMF_OK;
}

int cumf_hot_rows_assign(const cumf_hot_rows *h, cumf_node *d_R, int64_t nnz, void *stream) {
    TraceRange trace("hot rows: assign ratings to copies");
    if (!h || nnz < 0 || (nnz > 0 && !d_R)) return fail(CUMF_ERR_ARG, "hot_rows_assign: bad arguments");
    if (nnz == 0 || (h->hot_m == 0 && h->hot_n == 0)) return CUMF_OK;
    hot_assign_kernel<<<count_grid((uint64_t)nnz), kThreads, 0, (cudaStream_t)stream>>>(
        d_R, (uint64_t)nnz, h->hot_m ? h->tab_m : nullptr, (uint32_t)h->m, h->hot_n ? h->tab_n : nullptr,
        (uint32_t)h->n);
    CUMF_CUDA(cudaGetLastError());
    return CUMF_OK;
}

int cumf_hot_rows_spread(const cumf_hot_rows *h, void *d_P, void *d_Q, int k, int precision, void *stream) {
    if (!h || k < 1) return fail(CUMF_ERR_ARG, "hot_rows_spread: bad arguments");
    if (precision < CUMF_FP16 || precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    return merge_launch(h, d_P, d_Q, k, precision, 0, (cudaStream_t)stream);
}

int cumf_hot_rows_merge(const cumf_hot_rows *h, void *d_P, void *d_Q, int k, int precision, void *stream) {
    if (!h || k < 1) return fail(CUMF_ERR_ARG, "hot_rows_merge: bad arguments");
    if (precision < CUMF_FP16 || precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    return merge_launch(h, d_P, d_Q, k, precision, 1, (cudaStream_t)stream);
}

int cumf_hot_rows_free(cumf_hot_rows *h) {
    if (!h) return CUMF_OK;
    int cur = 0;
    const bool other = cudaGetDevice(&cur) == cudaSuccess && cur != h->device;
    if (other) cudaSetDevice(h->device);
    delete h;
    if (other) cudaSetDevice(cur);
    return CUMF_OK;
}

}  // extern "C"
