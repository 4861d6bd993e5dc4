// api_train.cpp - sgd_train orchestration (modes A, B, C), the RMSE evaluator entry
// points and the device-level wrappers of the C ABI.
//
// Mode A (u*v == 1, singleGPU/sgd_kernel.cu:212-248): the whole problem lives in HBM.  The
// raw records are copied once; stats, id shuffle, scaling, factor init, the SGD epochs and
// the fp32 export all run on the device, and only the final fp32 P and Q come back.
// Modes B and C (u*v > 1) keep the ratings and factors in host memory and stream blocks
// through the device (see stream_train below).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "cumf_sgd.h"
#include "glibc_shuffle.h"
#include "internal.h"
#include "train_common.h"

namespace cumf {

namespace {

void print_args(const cumf_params &p) {
    printf("k          :%d\n", p.k);
    printf("num_workers:%d\n", p.num_workers);
    printf("u_grid     :%d\n", p.u_grid);
    printf("v_grid     :%d\n", p.v_grid);
    printf("x_grid     :%d\n", p.x_grid);
    printf("y_grid     :%d\n", p.y_grid);
    printf("ux         :%d\n", p.ux);
    printf("vy         :%d\n", p.vy);
    printf("num_iters  :%d\n", p.num_iters);
    printf("gpu        :%d\n", p.gpu);
    printf("lambda_p   :%.5f\n", p.lambda_p);
    printf("lambda_q   :%.5f\n", p.lambda_q);
    printf("lrate      :%.5f\n", p.lrate);
    printf("alpha      :%.4f\n", p.alpha);
    printf("beta       :%.4f\n", p.beta);
}

// Per-epoch validation of the in-progress model against a raw test set on the device.
struct EpochEval {
    const cumf_problem *va = nullptr;
    DevBuf d_va, d_pf, d_qf, d_part, d_sum;
    int32_t m = 0, n = 0, k = 0;
    int init(const cumf_problem *v, int32_t m_, int32_t n_, int k_, cudaStream_t s) {
        va = v;
        m = m_;
        n = n_;
        k = k_;
        CUMF_CUDA(d_va.alloc(std::max<int64_t>(1, v->nnz) * sizeof(cumf_node)));
        if (v->nnz) CUMF_CUDA(cudaMemcpyAsync(d_va.p, v->R, v->nnz * sizeof(cumf_node), cudaMemcpyHostToDevice, s));
        CUMF_CUDA(d_pf.alloc((size_t)m * k * sizeof(float)));
        CUMF_CUDA(d_qf.alloc((size_t)n * k * sizeof(float)));
        CUMF_CUDA(d_part.alloc(rmse_blocks(v->nnz) * sizeof(double)));
        CUMF_CUDA(d_sum.alloc(sizeof(double)));
        return CUMF_OK;
    }
    // Exports the current factors exactly as the final model would be and evaluates.
    int eval(const void *P, const void *Q, int precision, const int32_t *pmap,
             const int32_t *qmap, float factor, float b, cudaStream_t s, double *rmse) {
        CUMF_CUDA(launch_export(P, precision, pmap, m, k, factor, d_pf.as<float>(), s));
        CUMF_CUDA(launch_export(Q, precision, qmap, n, k, factor, d_qf.as<float>(), s));
        CUMF_CUDA(launch_rmse(d_va.as<cumf_node>(), va->nnz, d_pf.as<float>(), m, d_qf.as<float>(),
                              n, k, b, d_part.as<double>(), d_sum.as<double>(), s));
        double sum = 0;
        CUMF_CUDA(cudaMemcpyAsync(&sum, d_sum.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        CUMF_CUDA(cudaStreamSynchronize(s));
        *rmse = va->nnz ? sqrt(sum / (double)va->nnz) : 0.0;
        return CUMF_OK;
    }
};

// ---- checkpoints (cumf_train_ckpt) ----------------------------------------------------------

struct CkptHeader {
    char magic[8];
    int32_t version, k, precision, workers, lanes, num_iters, epochs_done, m, n, tail_epochs, reserved;
    uint64_t seed;
    float lambda_p, lambda_q, alpha, beta, lrate, hot_rows;
    int64_t nnz, tail_start;
    uint64_t records_digest, bytes_p, bytes_q, payload_digest;
};
constexpr char kCkptMagic[8] = {'C', 'U', 'M', 'F', 'C', 'K', 'P', '1'};

// The copies of the most-rated rows of one training call.
struct HotRows {
    cumf_hot_rows *h = nullptr;
    HotRows() = default;
    HotRows(const HotRows &) = delete;
    HotRows &operator=(const HotRows &) = delete;
    ~HotRows() {
        if (h) cumf_hot_rows_free(h);
    }
};

struct PinnedHost {
    void *p = nullptr;
    ~PinnedHost() {
        if (p) cudaFreeHost(p);
    }
};

int payload_digest(const void *d_P, size_t bp, const void *d_Q, size_t bq, unsigned long long *d_dig, cudaStream_t s,
                   uint64_t *out) {
    unsigned long long a = 0, b = 0;
    CUMF_CUDA(launch_digest(d_P, bp, d_dig, s));
    CUMF_CUDA(cudaMemcpyAsync(&a, d_dig, sizeof(a), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    CUMF_CUDA(launch_digest(d_Q, bq, d_dig, s));
    CUMF_CUDA(cudaMemcpyAsync(&b, d_dig, sizeof(b), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    *out = (uint64_t)a ^ ((uint64_t)b * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull);
    return CUMF_OK;
}

int ckpt_write(const char *path, CkptHeader h, const void *d_P, const void *d_Q, unsigned long long *d_dig,
               cudaStream_t s) {
    if (int rc = payload_digest(d_P, h.bytes_p, d_Q, h.bytes_q, d_dig, s, &h.payload_digest)) return rc;
    PinnedHost buf;
    CUMF_CUDA(cudaMallocHost(&buf.p, h.bytes_p + h.bytes_q + 16));
    char *hp = static_cast<char *>(buf.p);
    CUMF_CUDA(cudaMemcpyAsync(hp, d_P, h.bytes_p, cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaMemcpyAsync(hp + h.bytes_p, d_Q, h.bytes_q, cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return fail(CUMF_ERR_IO, "cannot open " + tmp + " for writing");
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    ok = ok && fwrite(hp, 1, h.bytes_p + h.bytes_q, f) == h.bytes_p + h.bytes_q;
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        return fail(CUMF_ERR_IO, std::string("checkpoint write failed: ") + path);
    }
    return CUMF_OK;
}

// Loads a matching checkpoint into d_P / d_Q; *found = false when the file does not exist.
int ckpt_read(const char *path, const CkptHeader &want, void *d_P, void *d_Q, unsigned long long *d_dig,
              cudaStream_t s, int32_t *epochs_done, bool *found) {
    *found = false;
    FILE *f = fopen(path, "rb");
    if (!f) return CUMF_OK;
    *found = true;
    CkptHeader h;
    const bool got = fread(&h, sizeof(h), 1, f) == 1;
    auto bad = [&](const char *what) {
        fclose(f);
        return fail(CUMF_ERR_FORMAT, std::string("checkpoint ") + path + " does not match this run: " + what);
    };
    if (!got || memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) return bad("not a checkpoint file");
    if (h.k != want.k || h.precision != want.precision) return bad("k or precision");
    if (h.workers != want.workers || h.lanes != want.lanes) return bad("workers or lanes");
    if (h.seed != want.seed) return bad("seed");
    if (h.lambda_p != want.lambda_p || h.lambda_q != want.lambda_q || h.alpha != want.alpha || h.beta != want.beta ||
        h.lrate != want.lrate)
        return bad("lambda or learning-rate parameters");
    if (h.m != want.m || h.n != want.n || h.nnz != want.nnz || h.records_digest != want.records_digest)
        return bad("training ratings");
    if (h.tail_epochs != want.tail_epochs || h.tail_start != want.tail_start) return bad("fold-in epochs");
    if (h.reserved != want.reserved) return bad("schedule (batch-Hogwild or deterministic grid)");
    if (h.hot_rows != want.hot_rows) return bad("copies of the most-rated rows (hot_rows)");
    if (h.bytes_p != want.bytes_p || h.bytes_q != want.bytes_q) return bad("factor sizes");
    if (h.epochs_done < 0 || h.epochs_done > want.num_iters) return bad("more epochs done than this run has");
    PinnedHost buf;
    if (cudaMallocHost(&buf.p, h.bytes_p + h.bytes_q + 16) != cudaSuccess) {
        fclose(f);
        cudaGetLastError();
        return fail(CUMF_ERR_NOMEM, "cannot allocate pinned memory for the checkpoint");
    }
    char *hp = static_cast<char *>(buf.p);
    const bool full = fread(hp, 1, h.bytes_p + h.bytes_q, f) == h.bytes_p + h.bytes_q;
    fclose(f);
    if (!full) return fail(CUMF_ERR_FORMAT, std::string("checkpoint ") + path + " is truncated");
    CUMF_CUDA(cudaMemcpyAsync(d_P, hp, h.bytes_p, cudaMemcpyHostToDevice, s));
    CUMF_CUDA(cudaMemcpyAsync(d_Q, hp + h.bytes_p, h.bytes_q, cudaMemcpyHostToDevice, s));
    uint64_t dg = 0;
    if (int rc = payload_digest(d_P, h.bytes_p, d_Q, h.bytes_q, d_dig, s, &dg)) return rc;
    if (dg != h.payload_digest) return fail(CUMF_ERR_FORMAT, std::string("checkpoint ") + path + " fails its digest");
    *epochs_done = h.epochs_done;
    return CUMF_OK;
}

int train_mode_a(const cumf_problem *tr, const cumf_problem *va, const cumf_params &p,
                 int workers, int lanes, cumf_model *out, cumf_train_stats *st,
                 const cumf_model *init = nullptr, double *epoch_rmse = nullptr, double *epoch_ms = nullptr,
                 const cumf_checkpoint *ck = nullptr, int32_t *epochs_done = nullptr) {
    const double t0 = now_ms();
    TraceRange trace_prep("cumf_train: prep (H2D, stats, shuffle+scale, init)");
    const int64_t nnz = tr->nnz;
    const int32_t m = tr->m, n = tr->n;
    const int k = p.k;
    Stream stream;
    CUMF_CUDA(cudaStreamCreateWithFlags(&stream.s, cudaStreamNonBlocking));
    cudaStream_t s = stream.s;

    DevBuf d_R, d_part, d_small, d_pmap, d_qmap, d_P, d_Q, d_lr, d_status, d_pf, d_qf;
    CUMF_CUDA(d_R.alloc(std::max<int64_t>(1, nnz) * sizeof(cumf_node)));
    if (nnz) CUMF_CUDA(cudaMemcpyAsync(d_R.p, tr->R, nnz * sizeof(cumf_node), cudaMemcpyHostToDevice, s));
    const bool use_ck = ck && ck->path && ck->path[0];
    DevBuf d_dig;
    unsigned long long records_digest = 0;
    if (use_ck) {  // fingerprint of the caller's ratings, before they are permuted and scaled
        CUMF_CUDA(d_dig.alloc(sizeof(unsigned long long)));
        CUMF_CUDA(launch_digest(d_R.p, (uint64_t)nnz * sizeof(cumf_node), d_dig.as<unsigned long long>(), s));
        CUMF_CUDA(cudaMemcpyAsync(&records_digest, d_dig.p, sizeof(records_digest), cudaMemcpyDeviceToHost, s));
    }

    // collect_data on the device.
    Prepared pr;
    CUMF_CUDA(d_part.alloc(2 * stats_blocks(nnz) * sizeof(double)));
    CUMF_CUDA(d_small.alloc(4 * sizeof(double)));
    CUMF_CUDA(d_status.alloc(sizeof(int)));
    CUMF_CUDA(cudaMemsetAsync(d_status.p, 0, sizeof(int), s));
    CUMF_CUDA(launch_rating_stats(d_R.as<cumf_node>(), nnz, d_part.as<double>(), d_small.as<double>(), s));
    double sums[2] = {0, 0};
    CUMF_CUDA(cudaMemcpyAsync(sums, d_small.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));

    // Id maps on the host (sequential glibc stream) while the stats run.
    make_maps((uint32_t)p.seed, m, n, pr);
    CUMF_CUDA(d_pmap.alloc((size_t)m * sizeof(int32_t)));
    CUMF_CUDA(d_qmap.alloc((size_t)n * sizeof(int32_t)));
    CUMF_CUDA(cudaMemcpyAsync(d_pmap.p, pr.pmap.data(), (size_t)m * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    CUMF_CUDA(cudaMemcpyAsync(d_qmap.p, pr.qmap.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    finish_stats(sums[0], sums[1], nnz, pr);

    // shuffle_problem + scale_problem in one pass: r * (float)(1.0/scale) (sgd.cu:672).
    const float rscale = (float)(1.0 / pr.scale);
    CUMF_CUDA(launch_shuffle_scale(d_R.as<cumf_node>(), d_R.as<cumf_node>(), nnz, d_pmap.as<int32_t>(), m,
                                   d_qmap.as<int32_t>(), n, rscale, d_status.as<int>(), s));
    const float lambda_p = p.lambda_p / pr.scale, lambda_q = p.lambda_q / pr.scale;  // sgd.cu:673-674

    // Copies of the most-rated rows (batch-Hogwild only): laid out from the ratings' counts,
    // and every rating of such a row rewritten to name its copy.
    const int strata_g = p.deterministic > 0 ? strata_groups(nnz, p.deterministic) : 0;
    HotRows hot;
    int32_t m_rows = m, n_rows = n;
    if (strata_g == 0 && p.tail_epochs <= 0 && nnz > 0) {
        int dev_h = 0, sms_h = 0;
        CUMF_CUDA(cudaGetDevice(&dev_h));
        CUMF_CUDA(cudaDeviceGetAttribute(&sms_h, cudaDevAttrMultiProcessorCount, dev_h));
        const int64_t per_copy = hot_rows_per_copy(nnz, workers, k, p.precision, lanes, p.hot_rows, sms_h);
        if (per_copy > 0) {
            if (int rc = cumf_hot_rows_plan(d_R.as<cumf_node>(), nnz, m, n, per_copy, kHotMaxCopies, &hot.h, s))
                return rc;
            int32_t hm = 0, hn = 0;
            cumf_hot_rows_info(hot.h, &m_rows, &n_rows, &hm, &hn);
            if (hm + hn == 0) {
                cumf_hot_rows_free(hot.h);
                hot.h = nullptr;
            } else if (int rc = cumf_hot_rows_assign(hot.h, d_R.as<cumf_node>(), nnz, s)) {
                return rc;
            }
        }
    }

    // init_model: every row, including rows without ratings (sgd.cu:548-591).
    const int eb = elem_bytes(p.precision);
    CUMF_CUDA(d_P.alloc((size_t)m_rows * k * eb));
    CUMF_CUDA(d_Q.alloc((size_t)n_rows * k * eb));
    CUMF_CUDA(launch_init_factors(d_P.p, m, k, p.precision, p.seed, 1, s));
    CUMF_CUDA(launch_init_factors(d_Q.p, n, k, p.precision, p.seed, 2, s));
    if (init) {  // starting factors for the first init->m users and init->n items
        const float f0 = (float)sqrt(pr.scale);
        const int64_t mi = std::min<int64_t>(init->m, m), ni = std::min<int64_t>(init->n, n);
        DevBuf tmp;
        CUMF_CUDA(tmp.alloc((size_t)std::max(mi, ni) * k * sizeof(float)));
        const bool on_device = init->pinned == 2;  // P and Q are device addresses
        if (mi > 0) {
            const float *src = init->P;
            if (!on_device) {
                CUMF_CUDA(cudaMemcpyAsync(tmp.p, init->P, (size_t)mi * k * sizeof(float), cudaMemcpyHostToDevice, s));
                src = tmp.as<float>();
            }
            CUMF_CUDA(launch_import(src, d_pmap.as<int32_t>(), mi, k, f0, d_P.p, p.precision, s));
        }
        if (ni > 0) {
            CUMF_CUDA(cudaStreamSynchronize(s));  // tmp is reused
            const float *src = init->Q;
            if (!on_device) {
                CUMF_CUDA(cudaMemcpyAsync(tmp.p, init->Q, (size_t)ni * k * sizeof(float), cudaMemcpyHostToDevice, s));
                src = tmp.as<float>();
            }
            CUMF_CUDA(launch_import(src, d_qmap.as<int32_t>(), ni, k, f0, d_Q.p, p.precision, s));
        }
        CUMF_CUDA(cudaStreamSynchronize(s));
    }
    if (hot.h)
        if (int rc = cumf_hot_rows_spread(hot.h, d_P.p, d_Q.p, k, p.precision, s)) return rc;

    std::vector<float> lr(std::max(1, p.num_iters + 4));
    cumf_lr_schedule(p.alpha, p.beta, p.lrate, (int)lr.size(), lr.data());
    CUMF_CUDA(d_lr.alloc(lr.size() * sizeof(float)));
    CUMF_CUDA(cudaMemcpyAsync(d_lr.p, lr.data(), lr.size() * sizeof(float), cudaMemcpyHostToDevice, s));

    // Deterministic schedule: the shuffled, scaled ratings stably sorted into G x G blocks.
    DevBuf d_S, d_off;
    if (strata_g > 0 && nnz > 0) {
        CUMF_CUDA(d_S.alloc((size_t)nnz * sizeof(cumf_node)));
        CUMF_CUDA(d_off.alloc(((size_t)strata_g * strata_g + 1) * sizeof(unsigned long long)));
        if (int rc = strata_layout(d_R.as<cumf_node>(), nnz, strata_g, d_S.as<cumf_node>(),
                                   d_off.as<unsigned long long>(), s))
            return rc;
    }

    const float factor = (float)sqrt(pr.scale);  // scale_model (sgd.cu:598)
    // model->b (sgd.cu:679); an empty problem (0 / 0 in the reference) gets b = 0.
    const float b = nnz ? pr.ave / pr.std_dev : 0.f;
    EpochEval ev;
    const bool per_epoch = (p.verbose_epochs || epoch_rmse || epoch_ms) && va && va->nnz > 0;
    if (per_epoch) {
        if (int rc = ev.init(va, m, n, k, s)) return rc;
    }
    CUMF_CUDA(cudaStreamSynchronize(s));
    const double t1 = now_ms();
    trace_prep.end();

    // SGD epochs.
    TraceRange trace_epochs("cumf_train: epochs");
    Event e0, e1;
    CUMF_CUDA(e0.create());
    CUMF_CUDA(e1.create());
    int lanes_used = lanes;
    double train_ms = 0;
    // One launch per epoch by default.  The reference runs all epochs in one persistent
    // launch (sgd_kernel.cu:212-244); measured on GB300 at 52 workers per SM, that leaves the
    // test RMSE 0.002 (480,189 x 17,770, 99M ratings) to 0.03 (10,000 x 2,000, Zipf 1.0)
    // worse than an epoch boundary after every epoch, at the same speed, so it is an opt-in
    // (epochs_per_launch = N) that also needs every worker resident: with more workers than
    // one wave, later blocks would start after earlier blocks had run all epochs and would
    // apply the first epochs' learning rates last.
    int dev = 0, sms = 0;
    CUMF_CUDA(cudaGetDevice(&dev));
    CUMF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const bool one_wave = workers <= resident_workers(k, p.precision, lanes, sms);
    int per_launch = (per_epoch || !one_wave || p.tail_epochs > 0 || p.epochs_per_launch <= 0)
                         ? 1
                         : p.epochs_per_launch;
    const bool tail = p.tail_epochs > 0 && p.tail_start > 0 && p.tail_start < nnz;

    // Checkpoints: resume, then launches that end on multiples of `every`.
    CkptHeader ckh;
    memset(&ckh, 0, sizeof(ckh));
    int first_ep = 0, last_ep = p.num_iters;
    if (use_ck) {
        memcpy(ckh.magic, kCkptMagic, 8);
        ckh.version = 1;
        ckh.k = k;
        ckh.precision = p.precision;
        ckh.workers = workers;
        ckh.lanes = lanes;
        ckh.num_iters = p.num_iters;
        ckh.m = m;
        ckh.n = n;
        ckh.tail_epochs = p.tail_epochs;
        ckh.reserved = strata_g;  // the deterministic schedule's grid (0: batch-Hogwild)
        ckh.seed = p.seed;
        ckh.lambda_p = p.lambda_p;
        ckh.lambda_q = p.lambda_q;
        ckh.alpha = p.alpha;
        ckh.beta = p.beta;
        ckh.lrate = p.lrate;
        ckh.nnz = nnz;
        ckh.tail_start = p.tail_start;
        ckh.records_digest = records_digest;
        ckh.hot_rows = hot.h ? p.hot_rows : 0.f;
        ckh.bytes_p = (uint64_t)m_rows * k * eb;
        ckh.bytes_q = (uint64_t)n_rows * k * eb;
        if (ck->resume) {
            bool found = false;
            int32_t done = 0;
            if (int rc = ckpt_read(ck->path, ckh, d_P.p, d_Q.p, d_dig.as<unsigned long long>(), s, &done, &found))
                return rc;
            if (found) first_ep = done;
        }
        if (ck->every > 0) per_launch = std::min(per_launch, ck->every);
        if (ck->stop_after > 0) last_ep = std::min(last_ep, std::max(first_ep, (int)ck->stop_after));
    }
    CUMF_CUDA(cudaStreamSynchronize(s));
    // Epochs are launched back to back unless an evaluation or a checkpoint needs the factors
    // between them (a host wait after every epoch measured 14.2 ms per c2 epoch against 12.9).
    const bool sync_each = per_epoch || use_ck;
    if (!sync_each) CUMF_CUDA(cudaEventRecord(e0.e, s));
    for (int ep = first_ep; ep < last_ep;) {
        int cnt = std::min(per_launch, last_ep - ep);
        if (use_ck && ck->every > 0) cnt = std::min(cnt, ck->every - ep % ck->every);
        const cumf_node *R_ep = d_R.as<cumf_node>();
        int64_t nnz_ep = nnz;
        int workers_ep = workers;
        if (tail && ep < p.tail_epochs) {  // epochs over the tail of the rating array only,
            cnt = 1;                        // with at most one worker per 1024 of its ratings
            R_ep += p.tail_start;
            nnz_ep = nnz - p.tail_start;
            workers_ep = (int)std::min<int64_t>(workers, std::max<int64_t>(1, nnz_ep / 1024));
        }
        if (sync_each) CUMF_CUDA(cudaEventRecord(e0.e, s));
        Tuning tu;
        tu.lanes = lanes;
        tu.prefetch = p.prefetch;
        tu.hints = p.l2_hints;
        tu.ring = p.ring;
        tu.freeze_q = (tail && ep < p.tail_epochs) ? 1 : 0;  // fold-in: items stay as given
        tu.copies = hot.h ? 1 : 0;
        if (strata_g > 0) {
            if (nnz > 0)
                if (int rc = strata_epochs(d_S.as<cumf_node>(), d_off.as<unsigned long long>(), strata_g, d_P.p, m,
                                           d_Q.p, n, k, p.precision, lr.data(), ep, cnt, lambda_p, lambda_q, p.seed,
                                           d_status.as<int>(), s))
                    return rc;
        } else {
            CUMF_CUDA(launch_sgd_update(R_ep, nnz_ep, d_P.p, m_rows, d_Q.p, n_rows, k, p.precision, workers_ep, tu,
                                        d_lr.as<float>(), ep, cnt, lambda_p, lambda_q, p.seed, d_status.as<int>(), s,
                                        &lanes_used));
            if (hot.h)
                if (int rc = cumf_hot_rows_merge(hot.h, d_P.p, d_Q.p, k, p.precision, s)) return rc;
        }
        float ms = 0;
        if (sync_each) {
            CUMF_CUDA(cudaEventRecord(e1.e, s));
            CUMF_CUDA(cudaEventSynchronize(e1.e));
            CUMF_CUDA(cudaEventElapsedTime(&ms, e0.e, e1.e));
            train_ms += ms;
        }
        if (per_epoch) {
            double rmse = 0;
            if (int rc = ev.eval(d_P.p, d_Q.p, p.precision, d_pmap.as<int32_t>(), d_qmap.as<int32_t>(), factor, b, s, &rmse))
                return rc;
            if (epoch_rmse) epoch_rmse[ep] = rmse;
            if (epoch_ms) epoch_ms[ep] = train_ms;
            if (p.verbose_epochs) {
                printf("{\"epoch\": %d, \"train_ms\": %.3f, \"elapsed_ms\": %.3f, \"test_rmse\": %.6f}\n", ep + cnt,
                       ms, train_ms, rmse);
                fflush(stdout);
            }
        }
        ep += cnt;
        if (use_ck && ((ck->every > 0 && ep % ck->every == 0) || ep == last_ep)) {
            ckh.epochs_done = ep;
            if (int rc = ckpt_write(ck->path, ckh, d_P.p, d_Q.p, d_dig.as<unsigned long long>(), s)) return rc;
        }
    }
    if (!sync_each) CUMF_CUDA(cudaEventRecord(e1.e, s));
    if (epochs_done) *epochs_done = std::max(first_ep, last_ep);
    const int epochs_run = std::max(0, last_ep - first_ep);
    int status = 0;
    CUMF_CUDA(cudaMemcpyAsync(&status, d_status.p, sizeof(int), cudaMemcpyDeviceToHost, s));

    // Export: fp32, unscaled, un-permuted (transform_feature_vector + scale_model + shuffle_model),
    // into the ratings buffer when it is large enough (it is not read again).  The export
    // kernels and copies are queued behind the epochs, and the model's (pinned) host buffers
    // are allocated while the GPU still runs the epochs.
    const size_t pfb = (size_t)m * k * sizeof(float), qfb = (size_t)n * k * sizeof(float);
    float *pf = nullptr, *qf = nullptr;
    if (d_R.bytes >= pfb + qfb) {
        pf = d_R.as<float>();
        qf = pf + (size_t)m * k;
    } else {
        CUMF_CUDA(d_pf.alloc(pfb));
        CUMF_CUDA(d_qf.alloc(qfb));
        pf = d_pf.as<float>();
        qf = d_qf.as<float>();
    }
    CUMF_CUDA(launch_export(d_P.p, p.precision, d_pmap.as<int32_t>(), m, k, factor, pf, s));
    CUMF_CUDA(launch_export(d_Q.p, p.precision, d_qmap.as<int32_t>(), n, k, factor, qf, s));
    if (int rc = cumf_alloc_model(m, n, k, out)) return rc;
    out->b = b;
    cudaError_t ce = cudaMemcpyAsync(out->P, pf, pfb, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(out->Q, qf, qfb, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess && !sync_each) {
        ce = cudaEventSynchronize(e1.e);
        float ms = 0;
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0.e, e1.e);
        train_ms = ms;
    }
    const double t2 = now_ms();  // the epochs are done
    trace_epochs.end();
    TraceRange trace_export("cumf_train: export (fp32, unscale, unpermute, D2H)");
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) {
        cumf_free_model(out);
        return cuda_fail(ce, "epochs or model export");
    }
    if (status != 0) {
        cumf_free_model(out);
        return fail(CUMF_ERR_RANGE, "a rating index was outside the factor matrices");
    }
    const double t3 = now_ms();
    if (st) {
        st->prep_ms = t1 - t0;
        st->train_ms = train_ms;
        st->export_ms = t3 - t2;
        st->total_ms = t3 - t0;
        st->updates_per_sec = train_ms > 0 ? (double)nnz * epochs_run / (train_ms * 1e-3) : 0.0;
        st->samples_per_epoch = (int64_t)workers * batches_per_worker(nnz, workers) * 128;
        st->mean = pr.ave;
        st->std_dev = pr.std_dev;
        st->mode = 0;
        st->num_workers = strata_g > 0 ? strata_g : workers;  // deterministic: workers per stratum
        st->lanes = lanes_used;
        if (hot.h) cumf_hot_rows_info(hot.h, nullptr, nullptr, &st->hot_users, &st->hot_items);
        st->extra_rows = (m_rows - m) + (n_rows - n);
    }
    if (!p.quiet) {
        printf("update_per_sec:%f\n", train_ms > 0 ? (double)nnz * epochs_run / (train_ms * 1e-3) : 0.0);
        fflush(stdout);
    }
    return CUMF_OK;
}

}  // namespace

int stream_train(const cumf_problem *tr, const cumf_params &p, int workers, int lanes,
                 cumf_model *out, cumf_train_stats *st);

}  // namespace cumf

using namespace cumf;

extern "C" {

int cumf_device_info(int gpu, int *sm_count, int *cc_major, int *cc_minor) {
    if (int rc = select_device(gpu)) return rc;
    int dev = 0;
    CUMF_CUDA(cudaGetDevice(&dev));
    if (sm_count) CUMF_CUDA(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
    if (cc_major) CUMF_CUDA(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    if (cc_minor) CUMF_CUDA(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    return CUMF_OK;
}

int cumf_default_workers(int sm_count, int k, int precision, int lanes) {
    if (lanes == 0) lanes = default_lanes(k, precision);
    const int w = resident_workers(k, precision, lanes, sm_count);
    cudaGetLastError();
    return w > 0 ? w : 52 * sm_count;
}

int cumf_auto_workers(int64_t nnz, int sm_count, int k, int precision, int lanes) {
    // Whole waves of resident workers, at least three: blocks that finish early are replaced
    // by waiting blocks, which balances the epoch's tail (measured on c2: 13.4 ms per epoch
    // against 15.8 ms with one wave).  Every worker runs ceil(nnz / (W * 128)) batches, so an
    // epoch processes W * batches * 128 >= nnz samples: of 3 to 16 waves the count that
    // overshoots nnz least is taken (ties: more waves, a finer tail), keeping at least 8
    // batches per worker (c2: 8 waves, 0.55% extra samples, against 1.8% with 3 waves).
    // Small problems run fewer workers than three waves (fewer lost updates on shared rows).
    const int64_t resident = cumf_default_workers(sm_count, k, precision, lanes);
    const int64_t cap = nnz / (128 * 8);
    if (3 * resident > cap) return (int)std::max<int64_t>(1, cap);
    int64_t best_w = 3 * resident, best_samples = INT64_MAX;
    for (int waves = 3; waves <= 16; ++waves) {
        const int64_t w = waves * resident;
        const int64_t b = (nnz + w * 128 - 1) / (w * 128);
        if (b < 8 || w > 0x7fffffffll) break;
        if (w * b * 128 <= best_samples) {
            best_samples = w * b * 128;
            best_w = w;
        }
    }
    return (int)best_w;
}

// num_workers 0: cumf_auto_workers for the ratings of one grid block (the whole problem in
// mode A).
static int resolve_workers(const cumf_problem *tr, const cumf_params &p, int lanes) {
    if (p.num_workers > 0) return p.num_workers;
    int sms = 0;
    if (cumf_device_info(p.gpu, &sms, nullptr, nullptr) != CUMF_OK || sms <= 0) sms = 148;
    const int64_t blocks = (int64_t)std::max(1, p.ux) * std::max(1, p.vy);
    return cumf_auto_workers(std::max<int64_t>(1, tr->nnz / blocks), sms, p.k, p.precision, lanes);
}

int cumf_train(const cumf_problem *tr, const cumf_problem *va, const cumf_params *params,
               cumf_model *out, cumf_train_stats *stats) {
    if (!tr || !out) return fail(CUMF_ERR_ARG, "train: problem and model must not be NULL");
    if (tr->nnz < 0 || (tr->nnz > 0 && !tr->R) || tr->m < 1 || tr->n < 1)
        return fail(CUMF_ERR_ARG, "train: malformed problem");
    memset(out, 0, sizeof(*out));
    if (stats) memset(stats, 0, sizeof(*stats));
    if (int rc = check_params(params)) return rc;
    cumf_params p = *params;
    if (p.u_grid * p.v_grid == 1) p.x_grid = p.y_grid = 1;
    p.ux = p.u_grid * p.x_grid;
    p.vy = p.v_grid * p.y_grid;
    if (int rc = select_device(p.gpu)) return rc;
    const int lanes = p.lanes ? p.lanes : default_lanes(p.k, p.precision);
    p.num_workers = resolve_workers(tr, p, lanes);
    const int workers = p.num_workers;
    if (!p.quiet) {
        print_args(p);
        fflush(stdout);
    }
    if (p.ux * p.vy == 1) return train_mode_a(tr, va, p, workers, lanes, out, stats);
    return stream_train(tr, p, workers, lanes, out, stats);
}

int cumf_train_ex(const cumf_problem *tr, const cumf_problem *te, const cumf_params *params,
                  const cumf_model *init, cumf_model *out, cumf_train_stats *stats, double *epoch_rmse,
                  double *epoch_ms) {
    if (!tr || !out) return fail(CUMF_ERR_ARG, "train_ex: problem and model must not be NULL");
    if (tr->nnz < 0 || (tr->nnz > 0 && !tr->R) || tr->m < 1 || tr->n < 1)
        return fail(CUMF_ERR_ARG, "train_ex: malformed problem");
    memset(out, 0, sizeof(*out));
    if (stats) memset(stats, 0, sizeof(*stats));
    if (int rc = check_params(params)) return rc;
    cumf_params p = *params;
    if (p.u_grid * p.v_grid != 1) return fail(CUMF_ERR_ARG, "train_ex: only u = v = 1 (the whole problem in HBM)");
    p.x_grid = p.y_grid = 1;
    p.ux = p.vy = 1;
    if (init && (init->k != p.k || (init->m > 0 && !init->P) || (init->n > 0 && !init->Q)))
        return fail(CUMF_ERR_ARG, "train_ex: init model does not match k");
    if (int rc = select_device(p.gpu)) return rc;
    const int lanes = p.lanes ? p.lanes : default_lanes(p.k, p.precision);
    p.num_workers = resolve_workers(tr, p, lanes);
    if (!p.quiet) print_args(p);
    return train_mode_a(tr, te, p, p.num_workers, lanes, out, stats, init, epoch_rmse, epoch_ms);
}

int cumf_train_ckpt(const cumf_problem *tr, const cumf_problem *te, const cumf_params *params,
                    const cumf_checkpoint *ckpt, cumf_model *out, cumf_train_stats *stats, int32_t *epochs_done) {
    if (!tr || !out || !ckpt || !ckpt->path || !ckpt->path[0])
        return fail(CUMF_ERR_ARG, "train_ckpt: problem, model and checkpoint path must be given");
    if (ckpt->every < 0 || ckpt->stop_after < 0) return fail(CUMF_ERR_ARG, "train_ckpt: negative every or stop_after");
    if (tr->nnz < 0 || (tr->nnz > 0 && !tr->R) || tr->m < 1 || tr->n < 1)
        return fail(CUMF_ERR_ARG, "train_ckpt: malformed problem");
    memset(out, 0, sizeof(*out));
    if (stats) memset(stats, 0, sizeof(*stats));
    if (epochs_done) *epochs_done = 0;
    if (int rc = check_params(params)) return rc;
    cumf_params p = *params;
    if (p.u_grid * p.v_grid != 1) return fail(CUMF_ERR_ARG, "train_ckpt: checkpoints need u = v = 1 (the whole problem in HBM)");
    p.x_grid = p.y_grid = 1;
    p.ux = p.vy = 1;
    if (int rc = select_device(p.gpu)) return rc;
    const int lanes = p.lanes ? p.lanes : default_lanes(p.k, p.precision);
    p.num_workers = resolve_workers(tr, p, lanes);
    if (!p.quiet) print_args(p);
    return train_mode_a(tr, te, p, p.num_workers, lanes, out, stats, nullptr, nullptr, nullptr, ckpt, epochs_done);
}

int cumf_rmse(const cumf_problem *te, const cumf_model *model, double *out) {
    TraceRange trace("evaluate: RMSE");
    if (!te || !model || !out) return fail(CUMF_ERR_ARG, "rmse: NULL argument");
    if (te->nnz == 0) {  // calc_rmse returns 0 for an empty set (mf.cpp:3818-3819)
        *out = 0;
        return CUMF_OK;
    }
    if (!te->R || !model->P || !model->Q || model->k <= 0) return fail(CUMF_ERR_ARG, "rmse: malformed input");
    if (int rc = select_device(0)) return rc;
    Stream stream;
    CUMF_CUDA(cudaStreamCreateWithFlags(&stream.s, cudaStreamNonBlocking));
    DevBuf d_R, d_P, d_Q, d_part, d_sum;
    const size_t pb = (size_t)model->m * model->k * sizeof(float), qb = (size_t)model->n * model->k * sizeof(float);
    CUMF_CUDA(d_R.alloc(te->nnz * sizeof(cumf_node)));
    CUMF_CUDA(d_P.alloc(pb));
    CUMF_CUDA(d_Q.alloc(qb));
    CUMF_CUDA(d_part.alloc(rmse_blocks(te->nnz) * sizeof(double)));
    CUMF_CUDA(d_sum.alloc(sizeof(double)));
    CUMF_CUDA(cudaMemcpyAsync(d_R.p, te->R, te->nnz * sizeof(cumf_node), cudaMemcpyHostToDevice, stream.s));
    if (pb) CUMF_CUDA(cudaMemcpyAsync(d_P.p, model->P, pb, cudaMemcpyHostToDevice, stream.s));
    if (qb) CUMF_CUDA(cudaMemcpyAsync(d_Q.p, model->Q, qb, cudaMemcpyHostToDevice, stream.s));
    CUMF_CUDA(launch_rmse(d_R.as<cumf_node>(), te->nnz, d_P.as<float>(), model->m, d_Q.as<float>(), model->n,
                          model->k, model->b, d_part.as<double>(), d_sum.as<double>(), stream.s));
    double sum = 0;
    CUMF_CUDA(cudaMemcpyAsync(&sum, d_sum.p, sizeof(double), cudaMemcpyDeviceToHost, stream.s));
    CUMF_CUDA(cudaStreamSynchronize(stream.s));
    *out = sqrt(sum / (double)te->nnz);
    return CUMF_OK;
}

// ---- device-level wrappers ---------------------------------------------------------

int cumf_dev_init_factors(void *d_factors, int64_t rows, int k, int precision, uint64_t seed,
                          uint32_t tag, void *stream) {
    if (rows < 0 || k <= 0 || (rows > 0 && !d_factors)) return fail(CUMF_ERR_ARG, "init_factors: bad arguments");
    if (precision < CUMF_FP16 || precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    CUMF_CUDA(launch_init_factors(d_factors, rows, k, precision, seed, tag, (cudaStream_t)stream));
    return CUMF_OK;
}

int cumf_sgd_update(const cumf_node *d_R, int64_t nnz, void *d_P, int32_t m, void *d_Q, int32_t n,
                    int k, int precision, int num_workers, int lanes, const float *d_lr,
                    int first_epoch, int n_epochs, float lambda_p, float lambda_q, uint64_t seed,
                    int *d_status, void *stream) {
    cumf_tuning t;
    memset(&t, 0, sizeof(t));
    t.lanes = lanes;
    t.prefetch = -1;
    t.l2_hints = -1;
    return cumf_sgd_update_tuned(d_R, nnz, d_P, m, d_Q, n, k, precision, num_workers, &t, d_lr, first_epoch,
                                 n_epochs, lambda_p, lambda_q, seed, d_status, stream);
}

int cumf_sgd_update_tuned(const cumf_node *d_R, int64_t nnz, void *d_P, int32_t m, void *d_Q, int32_t n,
                          int k, int precision, int num_workers, const cumf_tuning *tuning, const float *d_lr,
                          int first_epoch, int n_epochs, float lambda_p, float lambda_q, uint64_t seed,
                          int *d_status, void *stream) {
    Tuning tu;
    if (tuning) {
        tu.lanes = tuning->lanes;
        tu.prefetch = tuning->prefetch;
        tu.hints = tuning->l2_hints;
        tu.ring = tuning->ring;
        tu.freeze_q = tuning->freeze_q;
        tu.copies = tuning->rows_copied;
    }
    const int lanes = tu.lanes;
    if (nnz < 0 || num_workers < 1 || first_epoch < 0 || n_epochs < 0 || m < 1 || n < 1)
        return fail(CUMF_ERR_ARG, "sgd_update: bad sizes");
    if (nnz > 0 && (!d_R || !d_P || !d_Q || !d_lr)) return fail(CUMF_ERR_ARG, "sgd_update: NULL pointer");
    if (!valid_k(k)) return fail(CUMF_ERR_ARG, "sgd_update: unsupported k " + std::to_string(k));
    if (precision < CUMF_FP16 || precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    if (lanes != 0 && !lanes_supported(k, precision, lanes)) return fail(CUMF_ERR_ARG, "unsupported lane count");
    if (batches_per_worker(nnz, num_workers) * 4 > 0x7fffffffll)
        return fail(CUMF_ERR_ARG, "sgd_update: too many batches per worker");
    CUMF_CUDA(launch_sgd_update(d_R, nnz, d_P, m, d_Q, n, k, precision, num_workers, tu, d_lr, first_epoch,
                                n_epochs, lambda_p, lambda_q, seed, d_status, (cudaStream_t)stream, nullptr));
    return CUMF_OK;
}

int cumf_dev_rating_stats(const cumf_node *d_R, int64_t nnz, double *mean, double *std_dev, void *stream) {
    if (nnz < 0 || (nnz > 0 && !d_R) || !mean || !std_dev) return fail(CUMF_ERR_ARG, "rating_stats: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf part, sum;
    CUMF_CUDA(part.alloc(2 * stats_blocks(nnz) * sizeof(double)));
    CUMF_CUDA(sum.alloc(2 * sizeof(double)));
    CUMF_CUDA(launch_rating_stats(d_R, nnz, part.as<double>(), sum.as<double>(), s));
    double h[2];
    CUMF_CUDA(cudaMemcpyAsync(h, sum.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    const double ex = nnz ? h[0] / nnz : 0.0, ex2 = nnz ? h[1] / nnz : 0.0;
    *mean = ex;
    *std_dev = sqrt(ex2 - ex * ex);
    return CUMF_OK;
}

int cumf_dev_shuffle_scale(const cumf_node *d_in, cumf_node *d_out, int64_t nnz, const int32_t *d_p_map,
                           int32_t m, const int32_t *d_q_map, int32_t n, float scale, int *d_status,
                           void *stream) {
    if (nnz < 0 || (nnz > 0 && (!d_in || !d_out))) return fail(CUMF_ERR_ARG, "shuffle_scale: bad arguments");
    CUMF_CUDA(launch_shuffle_scale(d_in, d_out, nnz, d_p_map, m, d_q_map, n, scale, d_status, (cudaStream_t)stream));
    return CUMF_OK;
}

int cumf_dev_export_factors(const void *d_in, int precision, const int32_t *d_map, int64_t rows, int k,
                            float factor, float *d_out, void *stream) {
    if (rows < 0 || k <= 0 || (rows > 0 && (!d_in || !d_out))) return fail(CUMF_ERR_ARG, "export: bad arguments");
    if (precision < CUMF_FP16 || precision > CUMF_FP16_SR) return fail(CUMF_ERR_ARG, "unknown precision");
    CUMF_CUDA(launch_export(d_in, precision, d_map, rows, k, factor, d_out, (cudaStream_t)stream));
    return CUMF_OK;
}

int cumf_dev_rmse(const cumf_node *d_R, int64_t nnz, const float *d_P, int32_t m, const float *d_Q, int32_t n,
                  int k, float b, double *out_rmse, void *stream) {
    if (nnz < 0 || k <= 0 || !out_rmse || (nnz > 0 && (!d_R || !d_P || !d_Q)))
        return fail(CUMF_ERR_ARG, "dev_rmse: bad arguments");
    if (nnz == 0) {
        *out_rmse = 0;
        return CUMF_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf part, sum;
    CUMF_CUDA(part.alloc(rmse_blocks(nnz) * sizeof(double)));
    CUMF_CUDA(sum.alloc(sizeof(double)));
    CUMF_CUDA(launch_rmse(d_R, nnz, d_P, m, d_Q, n, k, b, part.as<double>(), sum.as<double>(), s));
    double h = 0;
    CUMF_CUDA(cudaMemcpyAsync(&h, sum.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    *out_rmse = sqrt(h / (double)nnz);
    return CUMF_OK;
}

}  // extern "C"
