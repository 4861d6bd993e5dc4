// batch.cu - many independent factorizations in one persistent launch.
//
// Problems of uneven size (m, n, nnz) and factor length k in {32, 64, 128}, fp16 factors,
// share one launch: a grid of resident blocks whose G-lane worker groups (G = 8, 16 or 32,
// chosen by the autotuner) take tasks from a global counter.  A task is one Hogwild worker of one problem: it runs that worker's
// epochs of the launch in order, each its ceil(nnz/(W*128)) batches of 128 records exactly as
// in sgd_update.cu, so a problem never has more than W workers in flight and there is no
// barrier between epochs (as in the reference's persistent kernel).  The task table order is
// chosen by the autotuner.  Each lane owns k/G consecutive halves of a row (4 to 32 B).
// The launch (counter reset + kernel) can be captured in a CUDA graph and replayed.
// Problems may carry copies of their most-rated rows (hot_rows.cu); the batch then runs one
// launch per epoch and merges the copies between epochs, all inside the same graph.
// Autotuning times candidate schedules (lanes per worker, blocks per SM, workers per
// problem, task order) with an all-zero learning-rate table: the kernel then does the same loads and stores but
// writes back the values it read (p + 0 = p, exactly representable), so the factors are
// left bit for bit unchanged.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "cumf_sgd.h"
#include "device_common.cuh"
#include "internal.h"
#include "train_common.h"

namespace cumf {

namespace {

constexpr int kBT = 256;       // threads per block
constexpr int kBChunk = 32;    // records staged in shared memory at a time

struct BatchProblemDev {
    const cumf_node *R;
    uint64_t nnz;
    void *P;
    void *Q;
    uint32_t m, n;
    int k;
    int workers;
    int batches;
    float lp, lq;
    uint64_t seed;
    const float *lr;
};

struct BatchTask {
    int problem;
    int worker;
};

// A lane's slice of a row: E consecutive halves moved as NVEC vectors of type V.
template <int E>
struct LaneIO;
template <>
struct LaneIO<2> {
    using V = uint32_t;
    static constexpr int NVEC = 1;
};
template <>
struct LaneIO<4> {
    using V = uint2;
    static constexpr int NVEC = 1;
};
template <>
struct LaneIO<8> {
    using V = uint4;
    static constexpr int NVEC = 1;
};
template <>
struct LaneIO<16> {
    using V = uint4;
    static constexpr int NVEC = 2;
};

template <typename T>
__device__ __forceinline__ uint32_t &word(T &v, int w) {
    return reinterpret_cast<uint32_t *>(&v)[w];
}

__device__ __forceinline__ void bcp_async4(void *smem, const void *gmem) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// One worker's epoch on one problem: G lanes, E = k / G halves per lane (the lane's slice
// starts at element lane * E).  Dot product: lane partial in element order, then a shfl.xor
// butterfly over the G lanes (the order the oracle replays with lanes = G).
template <int G, int E>
__device__ void run_task(const BatchProblemDev &pr, int worker, int ep, int lane, unsigned gmask,
                         uint32_t (*s_rec)[3][kBChunk + 1], int *bad) {
    using IO = LaneIO<E>;
    using V = typename IO::V;
    constexpr int NVEC = IO::NVEC;
    constexpr int WPV = (int)(sizeof(V) / 4);  // 32-bit words (half pairs) per vector
    constexpr int ROWV = G * NVEC;             // vectors per row
    constexpr int WPL = kBChunk * 3 / G;       // staged record words per lane
    static_assert((kBChunk * 3) % G == 0, "record staging must split over the lanes");
    V *const P = reinterpret_cast<V *>(pr.P) + lane * NVEC;
    V *const Q = reinterpret_cast<V *>(pr.Q) + lane * NVEC;
    const uint32_t *const Rw = reinterpret_cast<const uint32_t *>(pr.R);
    const uint64_t nnz = pr.nnz;
    const float lr = __ldg(pr.lr + ep);
    const int chunks = pr.batches * (128 / kBChunk);
    auto fetch = [&](int t, int buf) {
        const uint64_t start = batch_start(pr.seed, ep, worker, t / (128 / kBChunk), nnz);
        uint64_t base = start + (uint64_t)((t % (128 / kBChunk)) * kBChunk);
        while (base >= nnz) base -= nnz;
#pragma unroll
        for (int i = 0; i < WPL; ++i) {
            const int w = lane + i * G;
            uint64_t rec = base + (uint64_t)(w / 3);
            while (rec >= nnz) rec -= nnz;
            bcp_async4(&s_rec[buf][w % 3][w / 3], Rw + rec * 3 + (w % 3));
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    auto load = [&](V (&dst)[NVEC], V *base, uint32_t row, bool ok) {
#pragma unroll
        for (int i = 0; i < NVEC; ++i) dst[i] = ok ? __ldcg(base + (uint64_t)row * ROWV + i) : V{};
    };
    fetch(0, 0);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncwarp(gmask);
    uint32_t u = s_rec[0][0][0], v = s_rec[0][1][0];
    bool ok = (u < pr.m) & (v < pr.n);
    V fp[NVEC], fq[NVEC];
    load(fp, P, u, ok);
    load(fq, Q, v, ok);
    for (int t = 0; t < chunks; ++t) {
        const int buf = t & 1;
        const bool has_next = t + 1 < chunks;
        if (has_next) fetch(t + 1, buf ^ 1);
#pragma unroll 1
        for (int j = 0; j < kBChunk; ++j) {
            uint32_t un = 0xffffffffu, vn = 0xffffffffu;
            if (j + 1 < kBChunk) {
                un = s_rec[buf][0][j + 1];
                vn = s_rec[buf][1][j + 1];
            } else if (has_next) {
                asm volatile("cp.async.wait_all;\n" ::: "memory");
                __syncwarp(gmask);
                un = s_rec[buf ^ 1][0][0];
                vn = s_rec[buf ^ 1][1][0];
            }
            const bool okn = (un < pr.m) & (vn < pr.n);
            V np[NVEC], nq[NVEC];
            load(np, P, un, okn);
            load(nq, Q, vn, okn);
            if (ok) {
                const float r = __uint_as_float(s_rec[buf][2][j]);
                float s = 0.f;
#pragma unroll
                for (int i = 0; i < NVEC; ++i)
#pragma unroll
                    for (int w = 0; w < WPV; ++w) {
                        const float2 pp = __half22float2(*reinterpret_cast<__half2 *>(&word(fp[i], w)));
                        const float2 qq = __half22float2(*reinterpret_cast<__half2 *>(&word(fq[i], w)));
                        s = __fmaf_rn(pp.x, qq.x, s);
                        s = __fmaf_rn(pp.y, qq.y, s);
                    }
#pragma unroll
                for (int o = G / 2; o >= 1; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                const float err = r - s;
                V wp[NVEC], wq[NVEC];
#pragma unroll
                for (int i = 0; i < NVEC; ++i)
#pragma unroll
                    for (int w = 0; w < WPV; ++w) {
                        const float2 pp = __half22float2(*reinterpret_cast<__half2 *>(&word(fp[i], w)));
                        const float2 qq = __half22float2(*reinterpret_cast<__half2 *>(&word(fq[i], w)));
                        const float px = __fmaf_rn(lr, __fmaf_rn(err, qq.x, -__fmul_rn(pr.lp, pp.x)), pp.x);
                        const float py = __fmaf_rn(lr, __fmaf_rn(err, qq.y, -__fmul_rn(pr.lp, pp.y)), pp.y);
                        const float qx = __fmaf_rn(lr, __fmaf_rn(err, pp.x, -__fmul_rn(pr.lq, qq.x)), qq.x);
                        const float qy = __fmaf_rn(lr, __fmaf_rn(err, pp.y, -__fmul_rn(pr.lq, qq.y)), qq.y);
                        __half2 hp = __floats2half2_rn(px, py), hq = __floats2half2_rn(qx, qy);
                        word(wp[i], w) = *reinterpret_cast<uint32_t *>(&hp);
                        word(wq[i], w) = *reinterpret_cast<uint32_t *>(&hq);
                    }
#pragma unroll
                for (int i = 0; i < NVEC; ++i) {
                    __stcg(P + (uint64_t)u * ROWV + i, wp[i]);
                    __stcg(Q + (uint64_t)v * ROWV + i, wq[i]);
                }
                if (un == u)
#pragma unroll
                    for (int i = 0; i < NVEC; ++i) np[i] = wp[i];
                if (vn == v)
#pragma unroll
                    for (int i = 0; i < NVEC; ++i) nq[i] = wq[i];
            } else {
                *bad = 1;
            }
#pragma unroll
            for (int i = 0; i < NVEC; ++i) {
                fp[i] = np[i];
                fq[i] = nq[i];
            }
            u = un;
            v = vn;
            ok = okn;
        }
        __syncwarp(gmask);
    }
}

// Persistent grid; each G-lane group takes tasks from the global counter.  G is the lanes
// per worker (8, 16 or 32; 32 needs every k >= 64).
template <int G>
__global__ void __launch_bounds__(kBT, 4)
batch_kernel(const BatchProblemDev *probs, const BatchTask *tasks, int tasks_per_epoch, int first_epoch, int n_epochs,
             int *counter, int *status) {
    constexpr int GPB = kBT / G;
    __shared__ uint32_t s_rec[GPB][2][3][kBChunk + 1];
    const int lane = threadIdx.x % G;
    const int gib = threadIdx.x / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const int leader = (threadIdx.x & 31) & ~(G - 1);
    int bad = 0;
    while (true) {
        int g = 0;
        if (lane == 0) g = atomicAdd(counter, 1);
        g = __shfl_sync(gmask, g, leader);
        if (g >= tasks_per_epoch) break;
        const BatchTask t = tasks[g];
        const BatchProblemDev pr = probs[t.problem];
        if (pr.nnz == 0 || pr.batches == 0) continue;
        for (int ep = first_epoch; ep < first_epoch + n_epochs; ++ep) {
            if (pr.k == 128 && G == 8) run_task<G, 16>(pr, t.worker, ep, lane, gmask, s_rec[gib], &bad);
            else if ((pr.k == 128 && G == 16) || (pr.k == 64 && G == 8))
                run_task<G, 8>(pr, t.worker, ep, lane, gmask, s_rec[gib], &bad);
            else if ((pr.k == 128 && G == 32) || (pr.k == 64 && G == 16) || (pr.k == 32 && G == 8))
                run_task<G, 4>(pr, t.worker, ep, lane, gmask, s_rec[gib], &bad);
            else if ((pr.k == 64 && G == 32) || (pr.k == 32 && G == 16))
                run_task<G, 2>(pr, t.worker, ep, lane, gmask, s_rec[gib], &bad);
            else
                bad = 1;
        }
    }
    if (bad && status && lane == 0) atomicExch(status, (int)CUMF_ERR_RANGE);
}

}  // namespace

struct Batch {
    std::vector<cumf_batch_problem> probs;
    std::vector<BatchProblemDev> dev_probs;
    cumf_batch_tuning tuning;
    DevBuf d_probs, d_probs_zero_lr, d_tasks, d_counter, d_status, d_zero_lr;
    int tasks_per_epoch = 0;
    int sm_count = 0;
    int64_t samples_per_epoch = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_first = -1, graph_n = -1;
    bool any_hot = false;  // a problem has row copies: one launch per epoch, merges between
    ~Batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

namespace {

int64_t work_of(const cumf_batch_problem &p) { return p.nnz * (int64_t)p.k; }

// Rebuilds worker counts, the device problem table and the task table for b->tuning.
int batch_plan(Batch *b) {
    const cumf_batch_tuning &t = b->tuning;
    const int nprob = (int)b->probs.size();
    b->dev_probs.resize(nprob);
    b->samples_per_epoch = 0;
    std::vector<int> workers(nprob);
    for (int i = 0; i < nprob; ++i) {
        const cumf_batch_problem &p = b->probs[i];
        int w = p.num_workers;
        if (w <= 0) {  // enough workers for ~batches_target batches each
            const int64_t target = std::max(1, t.batches_target);
            w = (int)std::max<int64_t>(1, (p.nnz + 128 * target - 1) / (128 * target));
        }
        workers[i] = w;
        BatchProblemDev &d = b->dev_probs[i];
        d.R = p.d_R;
        d.nnz = (uint64_t)p.nnz;
        d.P = p.d_P;
        d.Q = p.d_Q;
        d.m = (uint32_t)p.m;
        d.n = (uint32_t)p.n;
        if (p.hot) {  // ratings may name the copies' extra rows
            int32_t hm, hn, mr, nr;
            hot_rows_dims(p.hot, &hm, &hn, &mr, &nr);
            d.m = (uint32_t)mr;
            d.n = (uint32_t)nr;
        }
        d.k = p.k;
        d.workers = w;
        d.batches = (int)batches_per_worker(p.nnz, w);
        d.lp = p.lambda_p;
        d.lq = p.lambda_q;
        d.seed = p.seed;
        d.lr = p.d_lr;
        b->samples_per_epoch += (int64_t)w * d.batches * 128;
    }
    std::vector<int> order(nprob);
    std::iota(order.begin(), order.end(), 0);
    if (t.order == 2)  // largest problems first
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int c) { return work_of(b->probs[a]) > work_of(b->probs[c]); });
    std::vector<BatchTask> tasks;
    if (t.order == 1) {  // round robin across problems
        int maxw = 0;
        for (int i : order) maxw = std::max(maxw, workers[i]);
        for (int w = 0; w < maxw; ++w)
            for (int i : order)
                if (w < workers[i]) tasks.push_back({i, w});
    } else {
        for (int i : order)
            for (int w = 0; w < workers[i]; ++w) tasks.push_back({i, w});
    }
    b->tasks_per_epoch = (int)tasks.size();
    CUMF_CUDA(b->d_probs.alloc(std::max<size_t>(1, nprob) * sizeof(BatchProblemDev)));
    CUMF_CUDA(cudaMemcpy(b->d_probs.p, b->dev_probs.data(), nprob * sizeof(BatchProblemDev), cudaMemcpyHostToDevice));
    std::vector<BatchProblemDev> zl = b->dev_probs;
    for (BatchProblemDev &d : zl) d.lr = b->d_zero_lr.as<float>();
    CUMF_CUDA(b->d_probs_zero_lr.alloc(std::max<size_t>(1, nprob) * sizeof(BatchProblemDev)));
    CUMF_CUDA(cudaMemcpy(b->d_probs_zero_lr.p, zl.data(), nprob * sizeof(BatchProblemDev), cudaMemcpyHostToDevice));
    CUMF_CUDA(b->d_tasks.alloc(std::max<size_t>(1, tasks.size()) * sizeof(BatchTask)));
    CUMF_CUDA(cudaMemcpy(b->d_tasks.p, tasks.data(), tasks.size() * sizeof(BatchTask), cudaMemcpyHostToDevice));
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    b->graph_first = b->graph_n = -1;
    return CUMF_OK;
}

// Lanes per worker that every problem of the batch supports (k / lanes halves per lane, 2..16).
bool lanes_fit(const Batch *b, int lanes) {
    if (lanes != 8 && lanes != 16 && lanes != 32) return false;
    for (const cumf_batch_problem &p : b->probs)
        if (p.k / lanes < 2) return false;
    return true;
}

cudaError_t kernel_launch(Batch *b, bool zero_lr, int first_epoch, int n_epochs, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(b->d_counter.p, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    const int bps = std::max(1, std::min(4, b->tuning.blocks_per_sm));
    const BatchProblemDev *probs = zero_lr ? b->d_probs_zero_lr.as<BatchProblemDev>() : b->d_probs.as<BatchProblemDev>();
    const int grid = bps * b->sm_count;
    switch (b->tuning.lanes) {
        case 8:
            batch_kernel<8><<<grid, kBT, 0, s>>>(probs, b->d_tasks.as<BatchTask>(), b->tasks_per_epoch, first_epoch,
                                                  n_epochs, b->d_counter.as<int>(), b->d_status.as<int>());
            break;
        case 32:
            batch_kernel<32><<<grid, kBT, 0, s>>>(probs, b->d_tasks.as<BatchTask>(), b->tasks_per_epoch, first_epoch,
                                                   n_epochs, b->d_counter.as<int>(), b->d_status.as<int>());
            break;
        default:
            batch_kernel<16><<<grid, kBT, 0, s>>>(probs, b->d_tasks.as<BatchTask>(), b->tasks_per_epoch, first_epoch,
                                                   n_epochs, b->d_counter.as<int>(), b->d_status.as<int>());
            break;
    }
    return cudaGetLastError();
}

// The epochs of one run: one persistent launch, or with row copies one launch per epoch,
// each followed by the merge of every problem's copies (zero-learning-rate trials leave the
// copies equal, so they need no merge).
int batch_launch(Batch *b, bool zero_lr, int first_epoch, int n_epochs, cudaStream_t s) {
    if (zero_lr || !b->any_hot) {
        CUMF_CUDA(kernel_launch(b, zero_lr, first_epoch, n_epochs, s));
        return CUMF_OK;
    }
    for (int ep = first_epoch; ep < first_epoch + n_epochs; ++ep) {
        CUMF_CUDA(kernel_launch(b, false, ep, 1, s));
        for (const cumf_batch_problem &p : b->probs)
            if (p.hot)
                if (int rc = cumf_hot_rows_merge(p.hot, p.d_P, p.d_Q, p.k, CUMF_FP16, s)) return rc;
    }
    return CUMF_OK;
}

}  // namespace

}  // namespace cumf

using namespace cumf;

extern "C" {

int cumf_batch_create(const cumf_batch_problem *probs, int count, void **handle) {
    if (!probs || count <= 0 || !handle) return fail(CUMF_ERR_ARG, "batch_create: bad arguments");
    int max_epoch_index = 0;
    for (int i = 0; i < count; ++i) {
        const cumf_batch_problem &p = probs[i];
        if (p.k != 32 && p.k != 64 && p.k != 128)
            return fail(CUMF_ERR_ARG, "batch_create: k must be 32, 64 or 128 (problem " + std::to_string(i) + ")");
        if (p.nnz < 0 || p.m < 1 || p.n < 1 || (p.nnz > 0 && (!p.d_R || !p.d_P || !p.d_Q || !p.d_lr)))
            return fail(CUMF_ERR_ARG, "batch_create: malformed problem " + std::to_string(i));
        if (p.num_workers > 0 && batches_per_worker(p.nnz, p.num_workers) * 4 > 0x7fffffffll)
            return fail(CUMF_ERR_ARG, "batch_create: too many batches per worker");
        if (p.hot) {
            int32_t hm, hn, mr, nr;
            hot_rows_dims(p.hot, &hm, &hn, &mr, &nr);
            if (hm != p.m || hn != p.n)
                return fail(CUMF_ERR_ARG, "batch_create: row copies planned for another shape (problem " +
                                              std::to_string(i) + ")");
        }
        max_epoch_index = std::max(max_epoch_index, p.lr_len);
    }
    Batch *b = new Batch();
    b->probs.assign(probs, probs + count);
    for (const cumf_batch_problem &p : b->probs) b->any_hot = b->any_hot || p.hot != nullptr;
    b->tuning.batches_target = 16;
    b->tuning.order = 2;
    b->tuning.blocks_per_sm = 4;
    b->tuning.lanes = 16;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    auto bail = [&](int rc) {
        delete b;
        return rc;
    };
    if (cudaError_t e = b->d_counter.alloc(sizeof(int))) return bail(cuda_fail(e, "batch counter"));
    if (cudaError_t e = b->d_status.alloc(sizeof(int))) return bail(cuda_fail(e, "batch status"));
    if (cudaError_t e = b->d_zero_lr.alloc(std::max(1, max_epoch_index) * sizeof(float)))
        return bail(cuda_fail(e, "batch zero lr"));
    cudaMemset(b->d_status.p, 0, sizeof(int));
    cudaMemset(b->d_zero_lr.p, 0, std::max(1, max_epoch_index) * sizeof(float));
    if (int rc = batch_plan(b)) return bail(rc);
    *handle = b;
    return CUMF_OK;
}

int cumf_batch_destroy(void *handle) {
    delete static_cast<Batch *>(handle);
    return CUMF_OK;
}

int cumf_batch_set_tuning(void *handle, const cumf_batch_tuning *t) {
    Batch *b = static_cast<Batch *>(handle);
    if (!b || !t || t->order < 0 || t->order > 2 || t->batches_target < 1 || t->blocks_per_sm < 1 ||
        t->blocks_per_sm > 4)
        return fail(CUMF_ERR_ARG, "batch_set_tuning: bad tuning");
    cumf_batch_tuning c = *t;
    if (c.lanes == 0) c.lanes = 16;
    if (!lanes_fit(b, c.lanes))
        return fail(CUMF_ERR_ARG, "batch_set_tuning: lanes must be 8, 16 or 32 (32 needs every k >= 64)");
    b->tuning = c;
    return batch_plan(b);
}

int cumf_batch_get_info(void *handle, cumf_batch_tuning *t, int *tasks_per_epoch, int64_t *samples_per_epoch) {
    Batch *b = static_cast<Batch *>(handle);
    if (!b) return fail(CUMF_ERR_ARG, "batch_get_info: NULL handle");
    if (t) *t = b->tuning;
    if (tasks_per_epoch) *tasks_per_epoch = b->tasks_per_epoch;
    if (samples_per_epoch) *samples_per_epoch = b->samples_per_epoch;
    return CUMF_OK;
}

int cumf_batch_run(void *handle, int first_epoch, int n_epochs, int use_graph, void *stream) {
    Batch *b = static_cast<Batch *>(handle);
    if (!b || first_epoch < 0 || n_epochs < 0) return fail(CUMF_ERR_ARG, "batch_run: bad arguments");
    for (const cumf_batch_problem &p : b->probs)
        if (first_epoch + n_epochs > p.lr_len) return fail(CUMF_ERR_ARG, "batch_run: epochs beyond a problem's lr table");
    if (n_epochs == 0) return CUMF_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (!use_graph) return batch_launch(b, false, first_epoch, n_epochs, s);
    if (!b->exec || b->graph_first != first_epoch || b->graph_n != n_epochs) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        cudaStream_t cap;
        CUMF_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? batch_launch(b, false, first_epoch, n_epochs, cap) : CUMF_OK;
        cudaError_t e2 = cudaStreamEndCapture(cap, &b->graph);
        cudaStreamDestroy(cap);
        if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
        if (rc != CUMF_OK) return rc;
        if (e2 != cudaSuccess) return cuda_fail(e2, "batch graph end capture");
        CUMF_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->graph_first = first_epoch;
        b->graph_n = n_epochs;
    }
    CUMF_CUDA(cudaGraphLaunch(b->exec, s));
    return CUMF_OK;
}

int cumf_batch_status(void *handle, int *status) {
    Batch *b = static_cast<Batch *>(handle);
    if (!b || !status) return fail(CUMF_ERR_ARG, "batch_status: bad arguments");
    CUMF_CUDA(cudaMemcpy(status, b->d_status.p, sizeof(int), cudaMemcpyDeviceToHost));
    return CUMF_OK;
}

int cumf_batch_autotune(void *handle, void *stream, cumf_batch_tuning *best, double *best_ms) {
    Batch *b = static_cast<Batch *>(handle);
    if (!b) return fail(CUMF_ERR_ARG, "batch_autotune: NULL handle");
    cudaStream_t s = (cudaStream_t)stream;
    Event e0, e1;
    CUMF_CUDA(e0.create());
    CUMF_CUDA(e1.create());
    cumf_batch_tuning top = b->tuning;
    double top_ms = 1e30;
    // Time per sample of one epoch with a zero learning rate (factors unchanged), so schedules
    // with different budgets compare fairly.
    auto trial = [&](const cumf_batch_tuning &cand) -> int {
        b->tuning = cand;
        if (int rc = batch_plan(b)) return rc;
        if (int rc = batch_launch(b, true, 0, 1, s)) return rc;  // warm-up
        CUMF_CUDA(cudaEventRecord(e0.e, s));
        if (int rc = batch_launch(b, true, 0, 1, s)) return rc;
        CUMF_CUDA(cudaEventRecord(e1.e, s));
        CUMF_CUDA(cudaEventSynchronize(e1.e));
        float ms = 0;
        CUMF_CUDA(cudaEventElapsedTime(&ms, e0.e, e1.e));
        const double per = ms / (double)std::max<int64_t>(1, b->samples_per_epoch);
        if (per < top_ms) {
            top_ms = per;
            top = cand;
        }
        return CUMF_OK;
    };
    // Stage 1: lanes per worker x blocks per SM at the default budget and order; stage 2:
    // budget x task order at the chosen lanes and blocks.
    const int lanes_c[] = {8, 16, 32};
    const int occ[] = {3, 4};
    const int targets[] = {4, 8, 16, 32};
    const int orders[] = {0, 1, 2};
    cumf_batch_tuning cand = top;
    for (int g : lanes_c) {
        if (!lanes_fit(b, g)) continue;
        for (int bps : occ) {
            cand.lanes = g;
            cand.blocks_per_sm = bps;
            if (int rc = trial(cand)) return rc;
        }
    }
    const cumf_batch_tuning stage1 = top;
    for (int bt : targets)
        for (int o : orders) {
            cand = stage1;
            cand.batches_target = bt;
            cand.order = o;
            if (int rc = trial(cand)) return rc;
        }
    b->tuning = top;
    if (int rc = batch_plan(b)) return rc;
    if (best) *best = top;
    if (best_ms) *best_ms = top_ms * (double)b->samples_per_epoch;
    return CUMF_OK;
}

}  // extern "C"
