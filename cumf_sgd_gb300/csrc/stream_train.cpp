// stream_train.cpp - modes B and C of sgd_update_k128 (singleGPU/sgd_kernel.cu:249-690):
// the ratings and factors stay in host memory and u x v (mode B) or u x v x (x x y)
// (mode C) grid blocks are streamed through the device one at a time.
//
// Same as the reference:
//   - preparation order: stats, id maps, shuffle, grid_problem (exact in-place order), then
//     scale with block-local ids (sgd.cu:648-674);
//   - block order: the same rand() draws in the same order, continuing the glibc stream of
//     the id maps: mode B shuffles u, then v per u (sgd_kernel.cu:259-268); mode C shuffles
//     the u*v blocks, u, x, x*y and y per block (sgd_kernel.cu:406-432, the draws that do not
//     affect the order included), and runs each u*v block's x*y sub-blocks in natural order,
//     which is what its global_*_list indexing by sub-block id produces (:440-448);
//   - per block: one epoch of the update kernel over that block's ratings with budget
//     ceil(gridSize/(workers*128)) per worker (sgd_kernel.cu:198-208).
// Different by design:
//   - factor segments and rating blocks live in a two-slot device cache per kind; the next
//     block's copies run on a copy stream while the current block computes, ordered by
//     events (the reference issues the write-back D2H and the next H2D of the same buffer on
//     two unordered streams, sgd_kernel.cu:562-574, and synchronises the device every step);
//   - a block's sample stream is seeded with block_seed(seed, block id).
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <thread>
#include <vector>

#include "cumf_sgd.h"
#include "glibc_shuffle.h"
#include "internal.h"
#include "train_common.h"

namespace cumf {

namespace {

struct Step {
    int g;   // grid block id = gx * vy + gy
    int gx;  // P segment
    int gy;  // Q segment
};

// The block order of every epoch, drawing from `rng` exactly as the reference does.
std::vector<std::vector<Step>> block_schedule(const cumf_params &p, GlibcRand &rng) {
    const int ug = p.u_grid, vg = p.v_grid;
    const int xg = p.x_grid, yg = p.y_grid;
    const int vy = p.vy;
    const bool mode_c = xg * yg > 1;
    std::vector<int32_t> u_ids(ug), v_ids(vg), uv_ids(ug * vg), x_ids(xg), y_ids(yg), xy_ids(xg * yg);
    for (int i = 0; i < ug; ++i) u_ids[i] = i;
    for (int i = 0; i < vg; ++i) v_ids[i] = i;
    for (int i = 0; i < ug * vg; ++i) uv_ids[i] = i;
    for (int i = 0; i < xg; ++i) x_ids[i] = i;
    for (int i = 0; i < yg; ++i) y_ids[i] = i;
    for (int i = 0; i < xg * yg; ++i) xy_ids[i] = i;
    std::vector<std::vector<Step>> epochs(p.num_iters);
    for (int it = 0; it < p.num_iters; ++it) {
        if (mode_c) glibc_random_shuffle(uv_ids.data(), ug * vg, rng);
        glibc_random_shuffle(u_ids.data(), ug, rng);
        for (int u_ite = 0; u_ite < ug; ++u_ite) {
            if (!mode_c) glibc_random_shuffle(v_ids.data(), vg, rng);
            for (int v_ite = 0; v_ite < vg; ++v_ite) {
                int cu, cv;
                if (mode_c) {
                    cu = uv_ids[u_ite * vg + v_ite] / vg;
                    cv = uv_ids[u_ite * vg + v_ite] % vg;
                    glibc_random_shuffle(x_ids.data(), xg, rng);
                    glibc_random_shuffle(xy_ids.data(), xg * yg, rng);
                    for (int lx = 0; lx < xg; ++lx) glibc_random_shuffle(y_ids.data(), yg, rng);
                } else {
                    cu = u_ids[u_ite];
                    cv = v_ids[v_ite];
                }
                for (int sub = 0; sub < xg * yg; ++sub) {
                    const int gx = cu * xg + sub / yg, gy = cv * yg + sub % yg;
                    epochs[it].push_back(Step{gx * vy + gy, gx, gy});
                }
            }
        }
    }
    return epochs;
}

// Two device slots holding host segments `id` of `bytes` each (ratings: read-only; factor
// segments: written back when evicted).
struct SlotCache {
    struct Slot {
        int id = -1;
        DevBuf buf;
        cudaEvent_t ready = nullptr;  // H2D done
        cudaEvent_t idle = nullptr;   // last kernel using the slot done
        int64_t last_use = -1;
    };
    Slot slot[2];
    size_t seg_bytes = 0;
    bool writeback = false;

    int init(size_t bytes, bool wb) {
        seg_bytes = bytes;
        writeback = wb;
        for (Slot &s : slot) {
            CUMF_CUDA(s.buf.alloc(bytes));
            CUMF_CUDA(cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming));
            CUMF_CUDA(cudaEventCreateWithFlags(&s.idle, cudaEventDisableTiming));
        }
        return CUMF_OK;
    }
    ~SlotCache() {
        for (Slot &s : slot) {
            if (s.ready) cudaEventDestroy(s.ready);
            if (s.idle) cudaEventDestroy(s.idle);
        }
    }
    // Makes segment `id` resident; copies run on `copy` after the slot's last kernel.
    // host(id) gives the host address and size of segment id.
    template <typename HostFn>
    int acquire(int id, int64_t step, cudaStream_t copy, HostFn host, int *which) {
        for (int j = 0; j < 2; ++j) {
            if (slot[j].id == id) {
                slot[j].last_use = step;
                *which = j;
                return CUMF_OK;
            }
        }
        const int j = slot[0].last_use <= slot[1].last_use ? 0 : 1;  // least recently used
        Slot &s = slot[j];
        CUMF_CUDA(cudaStreamWaitEvent(copy, s.idle, 0));
        if (writeback && s.id >= 0) {
            size_t nb = 0;
            void *h = host(s.id, &nb);
            if (nb) CUMF_CUDA(cudaMemcpyAsync(h, s.buf.p, nb, cudaMemcpyDeviceToHost, copy));
        }
        size_t nb = 0;
        void *h = host(id, &nb);
        if (nb) CUMF_CUDA(cudaMemcpyAsync(s.buf.p, h, nb, cudaMemcpyHostToDevice, copy));
        CUMF_CUDA(cudaEventRecord(s.ready, copy));
        s.id = id;
        s.last_use = step;
        *which = j;
        return CUMF_OK;
    }
    template <typename HostFn>
    int flush(cudaStream_t copy, HostFn host) {
        for (Slot &s : slot) {
            if (!writeback || s.id < 0) continue;
            CUMF_CUDA(cudaStreamWaitEvent(copy, s.idle, 0));
            size_t nb = 0;
            void *h = host(s.id, &nb);
            if (nb) CUMF_CUDA(cudaMemcpyAsync(h, s.buf.p, nb, cudaMemcpyDeviceToHost, copy));
        }
        return CUMF_OK;
    }
};

struct PinnedBuf {
    void *p = nullptr;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
};

template <typename F>
void parallel_for(int64_t n, F f) {
    const int T = (int)std::max<unsigned>(1u, std::min<unsigned>(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            for (int64_t i = n * t / T; i < n * (t + 1) / T; ++i) f(i);
        });
    for (auto &x : th) x.join();
}

}  // namespace

int stream_train(const cumf_problem *tr, const cumf_params &p, int workers, int lanes,
                 cumf_model *out, cumf_train_stats *st) {
    const double t0 = now_ms();
    TraceRange trace_prep("cumf_train (streamed): prep (stats, shuffle, grid, scale, init)");
    const int64_t nnz = tr->nnz;
    const int32_t m = tr->m, n = tr->n;
    const int k = p.k;
    const int ux = p.ux, vy = p.vy;

    // Preparation on the host threads, equal to the reference's sequence collect_data,
    // shuffle_problem, grid_problem, scale_problem (sgd.cu:648-674) on a working copy:
    //   pass 1: rating sums (fp64 per chunk, added in chunk order) and the block id of every
    //           shuffled record, with per-block counts;
    //   grid_order: grid_problem's swap order replayed on the block ids;
    //   pass 2: the working copy gathered in that order from the caller's records, shuffled
    //           and scaled with block-local ids in the same step.
    Prepared pr;
    make_maps((uint32_t)p.seed, m, n, pr);
    const int32_t *pm = pr.pmap.data(), *qm = pr.qmap.data();
    const int64_t u_seg = ux == 1 ? m : (int64_t)ceil((double)m / ux);  // sgd.cu:419-426
    const int64_t v_seg = vy == 1 ? n : (int64_t)ceil((double)n / vy);
    const uint32_t us = (uint32_t)std::max<int64_t>(1, u_seg), vs = (uint32_t)std::max<int64_t>(1, v_seg);
    const int G = ux * vy;
    std::unique_ptr<int32_t[]> bid(new int32_t[(size_t)std::max<int64_t>(1, nnz)]);  // filled by the threads
    std::vector<double> p1(16, 0.0), p2(16, 0.0);
    std::vector<std::vector<int64_t>> part(16, std::vector<int64_t>(G, 0));
    std::vector<int> bad(16, 0);
    parallel_chunks(nnz, [&](int64_t a0, int64_t b0, int t) {
        double a1 = 0, a2 = 0;
        for (int64_t i = a0; i < b0; ++i) {
            const cumf_node x = tr->R[i];
            const double r = (double)x.r;
            a1 += r;
            a2 += r * r;
            if (x.u < 0 || x.u >= m || x.v < 0 || x.v >= n) {
                bad[t] = 1;
                bid[i] = 0;
                continue;
            }
            const int32_t g = (int32_t)(((uint32_t)pm[x.u] / us) * (uint32_t)vy + (uint32_t)qm[x.v] / vs);
            bid[i] = g;
            ++part[t][g];
        }
        p1[t] = a1;
        p2[t] = a2;
    });
    for (int t = 0; t < 16; ++t)
        if (bad[t]) return fail(CUMF_ERR_RANGE, "rating outside the grid");
    double s1 = 0, s2 = 0;
    for (int t = 0; t < 16; ++t) {
        s1 += p1[t];
        s2 += p2[t];
    }
    finish_stats(s1, s2, nnz, pr);
    std::vector<int64_t> grid_size(G, 0);
    for (int g = 0; g < G; ++g)
        for (int t = 0; t < 16; ++t) grid_size[g] += part[t][g];
    std::unique_ptr<int64_t[]> fin(new int64_t[(size_t)std::max<int64_t>(1, nnz)]);
    parallel_chunks(nnz, [&](int64_t a, int64_t b, int) {  // map the pages on all threads first
        if (b > a) memset(fin.get() + a, 0, (size_t)(b - a) * sizeof(int64_t));
    });
    grid_order(bid.get(), nnz, G, grid_size.data(), fin.get());
    bid.reset();
    PinnedBuf R_pin;
    CUMF_CUDA(cudaMallocHost(&R_pin.p, std::max<int64_t>(1, nnz) * sizeof(cumf_node)));
    cumf_node *R = static_cast<cumf_node *>(R_pin.p);
    const float rscale = (float)(1.0 / pr.scale);
    parallel_chunks(nnz, [&](int64_t a0, int64_t b0, int) {
        for (int64_t i = a0; i < b0; ++i) {
            const cumf_node x = tr->R[fin[i]];
            R[i].u = (int32_t)(pm[x.u] % u_seg);
            R[i].v = (int32_t)(qm[x.v] % v_seg);
            R[i].r = x.r * rscale;
        }
    });
    fin.reset();
    const float lambda_p = p.lambda_p / pr.scale, lambda_q = p.lambda_q / pr.scale;
    std::vector<int64_t> begin(ux * vy + 1, 0);
    for (int g = 0; g < ux * vy; ++g) begin[g + 1] = begin[g] + grid_size[g];

    Stream comp, copy;
    CUMF_CUDA(cudaStreamCreateWithFlags(&comp.s, cudaStreamNonBlocking));
    CUMF_CUDA(cudaStreamCreateWithFlags(&copy.s, cudaStreamNonBlocking));

    // Factors in host memory, in storage precision: ux*u_seg rows of P, vy*v_seg rows of Q,
    // initialised segment by segment on the device (sgd.cu:516-546).
    const int eb = elem_bytes(p.precision);
    const size_t pseg_bytes = (size_t)u_seg * k * eb, qseg_bytes = (size_t)v_seg * k * eb;
    PinnedBuf P_pin, Q_pin;
    CUMF_CUDA(cudaMallocHost(&P_pin.p, std::max<size_t>(1, pseg_bytes * ux)));
    CUMF_CUDA(cudaMallocHost(&Q_pin.p, std::max<size_t>(1, qseg_bytes * vy)));
    char *Ph = static_cast<char *>(P_pin.p), *Qh = static_cast<char *>(Q_pin.p);
    {
        DevBuf tmp;
        CUMF_CUDA(tmp.alloc(std::max(pseg_bytes, qseg_bytes)));
        for (int g = 0; g < ux; ++g) {
            CUMF_CUDA(launch_init_factors(tmp.p, u_seg, k, p.precision, p.seed, 1, comp.s, (uint64_t)g * u_seg * k));
            CUMF_CUDA(cudaMemcpyAsync(Ph + g * pseg_bytes, tmp.p, pseg_bytes, cudaMemcpyDeviceToHost, comp.s));
        }
        for (int g = 0; g < vy; ++g) {
            CUMF_CUDA(launch_init_factors(tmp.p, v_seg, k, p.precision, p.seed, 2, comp.s, (uint64_t)g * v_seg * k));
            CUMF_CUDA(cudaMemcpyAsync(Qh + g * qseg_bytes, tmp.p, qseg_bytes, cudaMemcpyDeviceToHost, comp.s));
        }
        CUMF_CUDA(cudaStreamSynchronize(comp.s));
    }

    std::vector<float> lr(std::max(1, p.num_iters + 4));
    cumf_lr_schedule(p.alpha, p.beta, p.lrate, (int)lr.size(), lr.data());
    DevBuf d_lr, d_status;
    CUMF_CUDA(d_lr.alloc(lr.size() * sizeof(float)));
    CUMF_CUDA(cudaMemcpy(d_lr.p, lr.data(), lr.size() * sizeof(float), cudaMemcpyHostToDevice));
    CUMF_CUDA(d_status.alloc(sizeof(int)));
    CUMF_CUDA(cudaMemset(d_status.p, 0, sizeof(int)));

    int64_t max_grid = 0;
    for (int64_t g : grid_size) max_grid = std::max(max_grid, g);
    SlotCache Rc, Pc, Qc;
    if (int rc = Rc.init(std::max<int64_t>(1, max_grid) * sizeof(cumf_node), false)) return rc;
    if (int rc = Pc.init(pseg_bytes, true)) return rc;
    if (int rc = Qc.init(qseg_bytes, true)) return rc;
    auto r_host = [&](int g, size_t *nb) -> void * {
        *nb = (size_t)grid_size[g] * sizeof(cumf_node);
        return R + begin[g];
    };
    auto p_host = [&](int g, size_t *nb) -> void * {
        *nb = pseg_bytes;
        return Ph + (size_t)g * pseg_bytes;
    };
    auto q_host = [&](int g, size_t *nb) -> void * {
        *nb = qseg_bytes;
        return Qh + (size_t)g * qseg_bytes;
    };

    const std::vector<std::vector<Step>> sched = block_schedule(p, pr.rng);
    const double t1 = now_ms();
    trace_prep.end();
    TraceRange trace_epochs("cumf_train (streamed): epochs (block copies + updates)");
    Tuning tu;
    tu.lanes = lanes;
    tu.prefetch = p.prefetch;
    tu.hints = p.l2_hints;
    tu.ring = p.ring;
    int64_t step = 0;
    for (int it = 0; it < p.num_iters; ++it) {
        for (const Step &sp : sched[it]) {
            int jr = 0, jp = 0, jq = 0;
            if (int rc = Rc.acquire(sp.g, step, copy.s, r_host, &jr)) return rc;
            if (int rc = Pc.acquire(sp.gx, step, copy.s, p_host, &jp)) return rc;
            if (int rc = Qc.acquire(sp.gy, step, copy.s, q_host, &jq)) return rc;
            CUMF_CUDA(cudaStreamWaitEvent(comp.s, Rc.slot[jr].ready, 0));
            CUMF_CUDA(cudaStreamWaitEvent(comp.s, Pc.slot[jp].ready, 0));
            CUMF_CUDA(cudaStreamWaitEvent(comp.s, Qc.slot[jq].ready, 0));
            CUMF_CUDA(launch_sgd_update(Rc.slot[jr].buf.as<cumf_node>(), grid_size[sp.g], Pc.slot[jp].buf.p,
                                        (int32_t)u_seg, Qc.slot[jq].buf.p, (int32_t)v_seg, k, p.precision, workers,
                                        tu, d_lr.as<float>(), it, 1, lambda_p, lambda_q, block_seed(p.seed, sp.g),
                                        d_status.as<int>(), comp.s, nullptr));
            CUMF_CUDA(cudaEventRecord(Rc.slot[jr].idle, comp.s));
            CUMF_CUDA(cudaEventRecord(Pc.slot[jp].idle, comp.s));
            CUMF_CUDA(cudaEventRecord(Qc.slot[jq].idle, comp.s));
            ++step;
        }
    }
    if (int rc = Pc.flush(copy.s, p_host)) return rc;
    if (int rc = Qc.flush(copy.s, q_host)) return rc;
    CUMF_CUDA(cudaStreamSynchronize(comp.s));
    CUMF_CUDA(cudaStreamSynchronize(copy.s));
    int status = 0;
    CUMF_CUDA(cudaMemcpy(&status, d_status.p, sizeof(int), cudaMemcpyDeviceToHost));
    const double t2 = now_ms();
    trace_epochs.end();
    if (status != 0) return fail(CUMF_ERR_RANGE, "a rating index was outside its block");
    TraceRange trace_export("cumf_train (streamed): export");

    // Export on the host: widen, unscale, un-permute (transform_half + scale_model +
    // shuffle_model); the model may not fit the device in these modes.
    if (int rc = cumf_alloc_model(m, n, k, out)) return rc;
    const float factor = (float)sqrt(pr.scale);
    out->b = tr->nnz ? pr.ave / pr.std_dev : 0.f;  // empty problem: b = 0 (0 / 0 in the reference)
    parallel_for(m, [&](int64_t o) {
        const int64_t src = pm[o];
        for (int j = 0; j < k; ++j) out->P[o * k + j] = store_to_float(Ph, src * k + j, p.precision) * factor;
    });
    parallel_for(n, [&](int64_t o) {
        const int64_t src = qm[o];
        for (int j = 0; j < k; ++j) out->Q[o * k + j] = store_to_float(Qh, src * k + j, p.precision) * factor;
    });
    const double t3 = now_ms();
    if (st) {
        st->prep_ms = t1 - t0;
        st->train_ms = t2 - t1;
        st->export_ms = t3 - t2;
        st->total_ms = t3 - t0;
        st->updates_per_sec = t2 > t1 ? (double)nnz * p.num_iters / ((t2 - t1) * 1e-3) : 0.0;
        int64_t samples = 0;
        for (int64_t gs : grid_size) samples += (int64_t)workers * batches_per_worker(gs, workers) * 128;
        st->samples_per_epoch = samples;
        st->mean = pr.ave;
        st->std_dev = pr.std_dev;
        st->mode = p.x_grid * p.y_grid > 1 ? 2 : 1;
        st->num_workers = workers;
        st->lanes = lanes;
    }
    if (!p.quiet) {
        printf("update_per_sec:%f\n", st ? st->updates_per_sec : 0.0);
        fflush(stdout);
    }
    return CUMF_OK;
}

}  // namespace cumf
