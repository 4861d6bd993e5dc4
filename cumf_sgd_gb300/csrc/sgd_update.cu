// sgd_update.cu - the batch-Hogwild SGD update kernel.
//
// Semantics follow sgd_k128_kernel_hogwild_warp32_lrate
// (singleGPU/sgd_k128_kernel_hogwild_warp32.h:3-104) launched by sgd_update_k128
// (singleGPU/sgd_kernel.cu:198-248):
//   - W workers; each does ceil(nnz/(W*128)) batches per epoch (sgd_kernel.cu:203);
//   - a batch is 128 consecutive records (start+i) % nnz from a uniform start (warp32.h:42-52);
//   - per record: e = r - <p_u, q_v>;  p <- p + lr (e q - lp p);  q <- q + lr (e p_old - lq q)
//     in fp32, stored back rounded to the storage type (warp32.h:85-99);
//   - lr = table[epoch] (warp32.h:32); no locks or atomics (Hogwild).
//
// GB300 layout: a worker is a group of G lanes (G = 4..32, a power of two) rather than a
// whole warp.  Each lane owns E = k/G consecutive elements of a row and moves them with
// 16-byte ld.global.cg / st.global.cg, so a k=128 fp16 row (256 B) is one vector per lane
// of a 16-lane group and two workers share a warp.  The dot product is a butterfly of
// shfl.xor within the group (every lane ends with the same bits).  The rows of record j+1
// are loaded while record j is reduced and updated (one-deep software pipeline); when
// record j+1 touches the row record j just wrote, the freshly computed values are forwarded
// instead, so each worker still applies its records strictly in order.  Records are staged
// 32 at a time through shared memory (coalesced 4-byte loads of the 12-byte records).
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_common.cuh"
#include "internal.h"

namespace cumf {

namespace {

constexpr int kBlock = 256;   // threads per block
constexpr int kMinBlocks = 4; // >= 1024 resident threads per SM (<= 64 registers)
constexpr int kDefaultPrefetch = 2;
constexpr int kDefaultHints = 1;
constexpr int kDefaultRing = 0;
constexpr int kBatch = 128;   // records per batch (update_vector_size, sgd_kernel.cu:198)
// Records staged in shared memory at a time: 32, or 16 for narrow groups (keeps the
// staging buffer of a 256-thread block under 27 KB).
__host__ __device__ constexpr int chunk_of(int lanes) { return lanes >= 8 ? 32 : 16; }

struct UpdateArgs {
    const cumf_node *R;
    uint64_t nnz;
    void *P;
    void *Q;
    uint32_t m, n;
    const float *lr;
    int first_epoch, n_epochs;
    int num_workers;
    int batches;
    float lambda_p, lambda_q;
    uint64_t seed;
    int *status;
    int prefetch;   // rows of record j+prefetch are pulled into L2 while record j runs (0 = off)
    int hints;      // 1 = L2 eviction hints (ratings evict_first, factor rows evict_last)
    int freeze_q;   // 1 = item rows are read but never written (user-side fold-in)
};

// Copy of a word the compiler cannot see through: the update phase re-widens the packed
// rows instead of keeping the dot phase's fp32 copies alive across the group reduction.
__device__ __forceinline__ uint4 opaque(uint4 w) {
    asm volatile("" : "+r"(w.x), "+r"(w.y), "+r"(w.z), "+r"(w.w));
    return w;
}

// The new rows of one record: p + lr*(e*q - lp*p) and q + lr*(e*p_old - lq*q)
// (warp32.h:89-99), in fp32, stored rounded to the storage type (stochastically when SR; the
// random bits of element pair h of word i of this lane are lowbias32(key + 2*pair) for p and
// lowbias32(key + 2*pair + 1) for q).  kUpdateQ = false (item rows frozen): wq is fq and none
// of q's arithmetic or random bits is computed.
template <class C, int NV, bool SR, bool kUpdateQ>
__device__ __forceinline__ void update_rows(const uint4 (&fp)[NV], const uint4 (&fq)[NV], uint4 (&wp)[NV],
                                            uint4 (&wq)[NV], float lr, float err, float lp, float lq, uint32_t key,
                                            int lane) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const uint4 fpi = opaque(fp[i]), fqi = opaque(fq[i]);
#pragma unroll
        for (int h = 0; h < C::kPairs; ++h) {
            const float2 pp = C::get(fpi, h), qq = C::get(fqi, h);
            const float px = __fmaf_rn(lr, __fmaf_rn(err, qq.x, -__fmul_rn(lp, pp.x)), pp.x);
            const float py = __fmaf_rn(lr, __fmaf_rn(err, qq.y, -__fmul_rn(lp, pp.y)), pp.y);
            if (kUpdateQ) {
                const float qx = __fmaf_rn(lr, __fmaf_rn(err, pp.x, -__fmul_rn(lq, qq.x)), qq.x);
                const float qy = __fmaf_rn(lr, __fmaf_rn(err, pp.y, -__fmul_rn(lq, qq.y)), qq.y);
                if (SR) {
                    const uint32_t pair = (uint32_t)(((lane * NV + i) * C::kPairs + h) * 2);
                    C::put_sr(wp[i], h, px, py, lowbias32(key + pair));
                    C::put_sr(wq[i], h, qx, qy, lowbias32(key + pair + 1u));
                } else {
                    C::put(wp[i], h, px, py);
                    C::put(wq[i], h, qx, qy);
                }
            } else if (SR) {
                const uint32_t pair = (uint32_t)(((lane * NV + i) * C::kPairs + h) * 2);
                C::put_sr(wp[i], h, px, py, lowbias32(key + pair));
            } else {
                C::put(wp[i], h, px, py);
            }
        }
        if (!kUpdateQ) wq[i] = fq[i];
    }
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, uint64_t pol) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int K, int KIND, int G, bool SR>
__global__ void __launch_bounds__(kBlock, kMinBlocks)
sgd_hogwild_kernel(const UpdateArgs a) {
    using C = Conv<KIND>;
    constexpr int SB = store_bytes(KIND);
    constexpr int ROW_WORDS = K * SB / 16;          // uint4 words per row
    constexpr int NV = ROW_WORDS / G;               // uint4 words per lane
    constexpr int GPB = kBlock / G;                 // groups (workers) per block
    constexpr int kChunk = chunk_of(G);
    constexpr int CPB = kBatch / kChunk;            // chunks per batch
    constexpr int WPL = kChunk * 3 / G;             // staged record words per lane
    static_assert(NV >= 1 && NV * G == ROW_WORDS, "lane split must cover the row");
    static_assert((kChunk * 3) % G == 0 && kBatch % kChunk == 0, "chunk must split evenly");

    // [group][buffer][field][record], padded so groups of one warp hit different banks.
    __shared__ uint32_t s_rec[GPB][2][3][kChunk + 1];

    const int lane = threadIdx.x % G;
    const int gib = threadIdx.x / G;
    const int worker = blockIdx.x * GPB + gib;
    if (worker >= a.num_workers) return;
    const unsigned gmask =
        (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));

    uint4 *const P = reinterpret_cast<uint4 *>(a.P) + lane * NV;
    uint4 *const Q = reinterpret_cast<uint4 *>(a.Q) + lane * NV;
    const uint32_t *const Rw = reinterpret_cast<const uint32_t *>(a.R);
    const uint64_t nnz = a.nnz;
    const float lp = a.lambda_p, lq = a.lambda_q;
    const int chunks = a.batches * CPB;
    const int pd = a.prefetch;
    const uint64_t pol_rec = l2_policy(a.hints != 0, false);
    const uint64_t pol_row = l2_policy(a.hints != 0, true);
    // Lanes whose 16-byte slice starts a 128-byte line issue the L2 prefetches.
    const bool pf_lane = ((lane * NV * 16) & 127) == 0;
    int bad = 0;

    for (int ep = a.first_epoch; ep < a.first_epoch + a.n_epochs; ++ep) {
        const float lr = __ldg(a.lr + ep);
        const uint32_t round_key = (uint32_t)(splitmix64(a.seed ^ (kTagRound << 48)) + (uint64_t)ep);

        // Asynchronous copy of the records of chunk t into buffer buf.
        auto fetch = [&](int t, int buf) {
            const uint64_t start = batch_start(a.seed, ep, worker, t / CPB, nnz);
            uint64_t base = start + (uint64_t)((t % CPB) * kChunk);
            while (base >= nnz) base -= nnz;  // start < nnz: wraps only when nnz < 128
#pragma unroll
            for (int i = 0; i < WPL; ++i) {
                const int word = lane + i * G;
                uint64_t rec = base + (uint64_t)(word / 3);
                while (rec >= nnz) rec -= nnz;
                cp_async4(&s_rec[gib][buf][word % 3][word / 3], Rw + rec * 3 + (word % 3), pol_rec);
            }
            cp_async_commit();
        };

        fetch(0, 0);
        cp_async_wait_all();
        __syncwarp(gmask);

        // Prologue: rows of the first record.
        uint32_t u = s_rec[gib][0][0][0], v = s_rec[gib][0][1][0];
        bool ok = (u < a.m) & (v < a.n);
        uint4 fp[NV], fq[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            fp[i] = ok ? ld_row_hint(P + (uint64_t)u * ROW_WORDS + i, pol_row) : make_uint4(0, 0, 0, 0);
            fq[i] = ok ? ld_row_hint(Q + (uint64_t)v * ROW_WORDS + i, pol_row) : make_uint4(0, 0, 0, 0);
        }

        for (int t = 0; t < chunks; ++t) {
            const int buf = t & 1;
            const bool has_next_chunk = (t + 1 < chunks);
            if (has_next_chunk) fetch(t + 1, buf ^ 1);

#pragma unroll 1
            for (int j = 0; j < kChunk; ++j) {
                // L2 prefetch of the rows of record j + pd (same or next chunk).
                if (pd > 0) {
                    const int jj = j + pd;
                    uint32_t pu = 0xffffffffu, pv = 0xffffffffu;
                    if (jj < kChunk) {
                        pu = s_rec[gib][buf][0][jj];
                        pv = s_rec[gib][buf][1][jj];
                    } else if (has_next_chunk && jj - kChunk < kChunk) {
                        if (jj == kChunk) {  // first look into the next chunk: wait for its copy
                            cp_async_wait_all();
                            __syncwarp(gmask);
                        }
                        pu = s_rec[gib][buf ^ 1][0][jj - kChunk];
                        pv = s_rec[gib][buf ^ 1][1][jj - kChunk];
                    }
                    if (pf_lane && pu < a.m && pv < a.n) {
                        prefetch_l2(P + (uint64_t)pu * ROW_WORDS);
                        prefetch_l2(Q + (uint64_t)pv * ROW_WORDS);
                    }
                }
                // Next record: same chunk, or the first record of the next chunk.
                uint32_t un = 0xffffffffu, vn = 0xffffffffu;
                if (j + 1 < kChunk) {
                    un = s_rec[gib][buf][0][j + 1];
                    vn = s_rec[gib][buf][1][j + 1];
                } else if (has_next_chunk) {
                    cp_async_wait_all();
                    __syncwarp(gmask);
                    un = s_rec[gib][buf ^ 1][0][0];
                    vn = s_rec[gib][buf ^ 1][1][0];
                }
                const bool okn = (un < a.m) & (vn < a.n);
                uint4 np[NV], nq[NV];
#pragma unroll
                for (int i = 0; i < NV; ++i) {
                    np[i] = okn ? ld_row_hint(P + (uint64_t)un * ROW_WORDS + i, pol_row) : make_uint4(0, 0, 0, 0);
                    nq[i] = okn ? ld_row_hint(Q + (uint64_t)vn * ROW_WORDS + i, pol_row) : make_uint4(0, 0, 0, 0);
                }

                if (ok) {
                    const float r = __uint_as_float(s_rec[gib][buf][2][j]);
                    // Lane partial dot in element order, then the group butterfly.
                    float s = 0.f;
#pragma unroll
                    for (int i = 0; i < NV; ++i) {
#pragma unroll
                        for (int h = 0; h < C::kPairs; ++h) {
                            const float2 pp = C::get(fp[i], h), qq = C::get(fq[i], h);
                            s = __fmaf_rn(pp.x, qq.x, s);
                            s = __fmaf_rn(pp.y, qq.y, s);
                        }
                    }
#pragma unroll
                    for (int o = G / 2; o >= 1; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                    const float err = r - s;
                    uint32_t key = 0;
                    if (SR) {
                        const uint32_t sample = (uint32_t)worker * (uint32_t)(chunks * kChunk) +
                                                (uint32_t)(t * kChunk + j);
                        key = round_key ^ lowbias32(sample);
                    }
                    uint4 wp[NV], wq[NV];
                    // Frozen item rows: the stochastic-rounding kernels skip q's arithmetic and
                    // random bits; the others compute q and keep the old row (fewer registers).
                    if (SR && a.freeze_q) {
                        update_rows<C, NV, SR, false>(fp, fq, wp, wq, lr, err, lp, lq, key, lane);
                    } else {
                        update_rows<C, NV, SR, true>(fp, fq, wp, wq, lr, err, lp, lq, key, lane);
                        if (a.freeze_q) {
#pragma unroll
                            for (int i = 0; i < NV; ++i) wq[i] = fq[i];
                        }
                    }
#pragma unroll
                    for (int i = 0; i < NV; ++i) {
                        st_row_hint(P + (uint64_t)u * ROW_WORDS + i, wp[i], pol_row);
                        if (!a.freeze_q) st_row_hint(Q + (uint64_t)v * ROW_WORDS + i, wq[i], pol_row);
                    }
                    // Forward the fresh rows when the next record reuses them (its loads
                    // were issued before these stores).
                    if (un == u) {
#pragma unroll
                        for (int i = 0; i < NV; ++i) np[i] = wp[i];
                    }
                    if (vn == v) {
#pragma unroll
                        for (int i = 0; i < NV; ++i) nq[i] = wq[i];
                    }
                } else {
                    bad = 1;
                }
#pragma unroll
                for (int i = 0; i < NV; ++i) {
                    fp[i] = np[i];
                    fq[i] = nq[i];
                }
                u = un;
                v = vn;
                ok = okn;
            }
            __syncwarp(gmask);  // buffer `buf` is refilled by the next iteration's fetch
        }
    }
    if (bad && a.status != nullptr && lane == 0) atomicExch(a.status, (int)CUMF_ERR_RANGE);
}


// ---- deeper pipeline: rows staged asynchronously through a shared-memory ring ----------
//
// Same semantics as sgd_hogwild_kernel, with D records' rows in flight per worker instead
// of one and no registers held for them: the rows of record x+D-1 are copied (cp.async,
// 16 bytes per lane, L2 only) into ring slot (x+D-1) % D while record x is computed.  Each
// lane only ever reads back its own slices, so the copy needs no cross-lane handoff.
// In-order semantics per worker: a record whose row was written by one of the D-1 records
// processed after its copy was issued takes the row from the previous record's registers
// (distance 1) or re-reads it from global memory (distance 2..D-1).
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, uint64_t pol) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "l"(pol)
                 : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int kRingDepth = 4;
constexpr int kRingMinBlocks = 4;

template <int K, int KIND, int G, int D>
struct RingLayout {
    static constexpr int SB = store_bytes(KIND);
    static constexpr int ROW_WORDS = K * SB / 16;
    static constexpr int GPB = kBlock / G;
    static constexpr int kChunk = chunk_of(G);
    static constexpr size_t rec_bytes = (size_t)GPB * 2 * 3 * (kChunk + 1) * 4;
    static constexpr size_t rec_bytes_aligned = (rec_bytes + 15) / 16 * 16;
    static constexpr size_t ring_bytes = (size_t)GPB * D * 2 * ROW_WORDS * 16;
    static constexpr size_t smem = rec_bytes_aligned + ring_bytes;
};

template <int K, int KIND, int G, bool SR, int D>
__global__ void __launch_bounds__(kBlock, kRingMinBlocks)
sgd_ring_kernel(const UpdateArgs a) {
    using C = Conv<KIND>;
    using L = RingLayout<K, KIND, G, D>;
    constexpr int ROW_WORDS = L::ROW_WORDS;
    constexpr int NV = ROW_WORDS / G;
    constexpr int GPB = L::GPB;
    constexpr int kChunk = L::kChunk;
    constexpr int CPB = kBatch / kChunk;
    constexpr int WPL = kChunk * 3 / G;
    static_assert(NV >= 1 && NV * G == ROW_WORDS, "lane split must cover the row");
    static_assert(kChunk >= 2 * D - 1, "a staged chunk must land before its first use");

    extern __shared__ __align__(16) unsigned char smem_raw[];
    typedef uint32_t RecBuf[2][3][kChunk + 1];
    RecBuf *s_rec = reinterpret_cast<RecBuf *>(smem_raw);

    const int lane = threadIdx.x % G;
    const int gib = threadIdx.x / G;
    const int worker = blockIdx.x * GPB + gib;
    if (worker >= a.num_workers) return;
    const unsigned gmask =
        (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    uint4 *const ring = reinterpret_cast<uint4 *>(smem_raw + L::rec_bytes_aligned) +
                        (size_t)gib * D * 2 * ROW_WORDS + lane * NV;

    uint4 *const P = reinterpret_cast<uint4 *>(a.P) + lane * NV;
    uint4 *const Q = reinterpret_cast<uint4 *>(a.Q) + lane * NV;
    const uint32_t *const Rw = reinterpret_cast<const uint32_t *>(a.R);
    const uint64_t nnz = a.nnz;
    const float lp = a.lambda_p, lq = a.lambda_q;
    const int chunks = a.batches * CPB;
    const int total = chunks * kChunk;
    const uint64_t pol_rec = l2_policy(a.hints != 0, false);
    const uint64_t pol_row = l2_policy(a.hints != 0, true);
    int bad = 0;

    for (int ep = a.first_epoch; ep < a.first_epoch + a.n_epochs; ++ep) {
        const float lr = __ldg(a.lr + ep);
        const uint32_t round_key = (uint32_t)(splitmix64(a.seed ^ (kTagRound << 48)) + (uint64_t)ep);

        auto fetch = [&](int t) {  // records of chunk t into buffer t & 1 (copies join the next group)
            const uint64_t start = batch_start(a.seed, ep, worker, t / CPB, nnz);
            uint64_t base = start + (uint64_t)((t % CPB) * kChunk);
            while (base >= nnz) base -= nnz;
#pragma unroll
            for (int i = 0; i < WPL; ++i) {
                const int word = lane + i * G;
                uint64_t rec = base + (uint64_t)(word / 3);
                while (rec >= nnz) rec -= nnz;
                cp_async4(&s_rec[gib][t & 1][word % 3][word / 3], Rw + rec * 3 + (word % 3), pol_rec);
            }
        };
        auto rec_field = [&](int x, int f) -> uint32_t { return s_rec[gib][(x / kChunk) & 1][f][x % kChunk]; };
        auto issue = [&](int y) {  // rows of record y into slot y % D; always commits one group
            if (y < total) {
                const uint32_t uy = rec_field(y, 0), vy = rec_field(y, 1);
                if ((uy < a.m) & (vy < a.n)) {
                    uint4 *slot = ring + (size_t)(y % D) * 2 * ROW_WORDS;
#pragma unroll
                    for (int i = 0; i < NV; ++i) {
                        cp_async16(slot + i, P + (uint64_t)uy * ROW_WORDS + i, pol_row);
                        cp_async16(slot + ROW_WORDS + i, Q + (uint64_t)vy * ROW_WORDS + i, pol_row);
                    }
                }
            }
            cp_async_commit();
        };

        fetch(0);
        cp_async_commit();
        cp_async_wait_all();
        __syncwarp(gmask);
        if (chunks > 1) fetch(1);  // joins the first row group below
#pragma unroll 1
        for (int y = 0; y < D - 1; ++y) issue(y);

        uint32_t pu[D - 1], pv[D - 1];
#pragma unroll
        for (int i = 0; i < D - 1; ++i) pu[i] = pv[i] = 0xffffffffu;
        uint4 wp[NV], wq[NV];  // rows written by the previous record
#pragma unroll
        for (int i = 0; i < NV; ++i) wp[i] = wq[i] = make_uint4(0, 0, 0, 0);

#pragma unroll 1
        for (int x = 0; x < total; ++x) {
            const int t = x / kChunk, j = x % kChunk;
            if (j == 0 && t >= 1) {
                __syncwarp(gmask);  // everyone is done with chunk t-1's buffer
                if (t + 1 < chunks) fetch(t + 1);
            }
            if (j == kChunk - D + 1 && t + 1 < chunks) __syncwarp(gmask);  // chunk t+1 visible to all lanes
            issue(x + D - 1);
            cp_async_wait_group<D - 1>();  // this lane's slices of record x have landed

            const uint32_t u = rec_field(x, 0), v = rec_field(x, 1);
            const bool ok = (u < a.m) & (v < a.n);
            if (ok) {
                const float r = __uint_as_float(rec_field(x, 2));
                const uint4 *slot = ring + (size_t)(x % D) * 2 * ROW_WORDS;
                bool p_reload = false, q_reload = false;
#pragma unroll
                for (int i = 1; i < D - 1; ++i) {
                    p_reload |= (u == pu[i]);
                    q_reload |= (v == pv[i]);
                }
                uint4 fp[NV], fq[NV];
#pragma unroll
                for (int i = 0; i < NV; ++i) {
                    fp[i] = (u == pu[0]) ? wp[i] : p_reload ? ld_row(P + (uint64_t)u * ROW_WORDS + i) : slot[i];
                    fq[i] = (v == pv[0]) ? wq[i] : q_reload ? ld_row(Q + (uint64_t)v * ROW_WORDS + i) : slot[ROW_WORDS + i];
                }
                float s = 0.f;
#pragma unroll
                for (int i = 0; i < NV; ++i) {
#pragma unroll
                    for (int h = 0; h < C::kPairs; ++h) {
                        const float2 pp = C::get(fp[i], h), qq = C::get(fq[i], h);
                        s = __fmaf_rn(pp.x, qq.x, s);
                        s = __fmaf_rn(pp.y, qq.y, s);
                    }
                }
#pragma unroll
                for (int o = G / 2; o >= 1; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
                const float err = r - s;
                uint32_t key = 0;
                if (SR) key = round_key ^ lowbias32((uint32_t)worker * (uint32_t)total + (uint32_t)x);
                if (SR && a.freeze_q) {
                    update_rows<C, NV, SR, false>(fp, fq, wp, wq, lr, err, lp, lq, key, lane);
                } else {
                    update_rows<C, NV, SR, true>(fp, fq, wp, wq, lr, err, lp, lq, key, lane);
                    if (a.freeze_q) {
#pragma unroll
                        for (int i = 0; i < NV; ++i) wq[i] = fq[i];
                    }
                }
#pragma unroll
                for (int i = 0; i < NV; ++i) {
                    st_row_hint(P + (uint64_t)u * ROW_WORDS + i, wp[i], pol_row);
                    if (!a.freeze_q) st_row_hint(Q + (uint64_t)v * ROW_WORDS + i, wq[i], pol_row);
                }
            } else {
                bad = 1;
            }
#pragma unroll
            for (int i = D - 2; i >= 1; --i) {
                pu[i] = pu[i - 1];
                pv[i] = pv[i - 1];
            }
            pu[0] = ok ? u : 0xffffffffu;
            pv[0] = ok ? v : 0xffffffffu;
        }
        cp_async_wait_all();
        __syncwarp(gmask);
    }
    if (bad && a.status != nullptr && lane == 0) atomicExch(a.status, (int)CUMF_ERR_RANGE);
}

using KernelFn = void (*)(const UpdateArgs);

struct KernelEntry {
    int k, kind, lanes;
    bool sr;
    KernelFn fn;
    KernelFn ring;        // deeper-pipeline variant (nullptr where not built)
    size_t ring_smem;     // its dynamic shared memory per block
};

#define CUMF_K(K, KIND, G, SR) {K, KIND, G, SR, &sgd_hogwild_kernel<K, KIND, G, SR>, \
    &sgd_ring_kernel<K, KIND, G, SR, kRingDepth>, RingLayout<K, KIND, G, kRingDepth>::smem}
#define CUMF_K_ALL_G(K, KIND, SR, G1, G2) CUMF_K(K, KIND, G1, SR), CUMF_K(K, KIND, G2, SR)

// For each (k, storage) two lane widths: one 16-byte word per lane, or two.
const KernelEntry kKernels[] = {
    // fp16 (rows of 2k bytes)
    CUMF_K(32, kHalf, 4, false),
    CUMF_K_ALL_G(64, kHalf, false, 8, 4),
    CUMF_K_ALL_G(128, kHalf, false, 16, 8),
    CUMF_K_ALL_G(256, kHalf, false, 32, 16),
    CUMF_K(32, kHalf, 4, true),
    CUMF_K_ALL_G(64, kHalf, true, 8, 4),
    CUMF_K_ALL_G(128, kHalf, true, 16, 8),
    CUMF_K_ALL_G(256, kHalf, true, 32, 16),
    // bf16
    CUMF_K(32, kBf16, 4, false),
    CUMF_K_ALL_G(64, kBf16, false, 8, 4),
    CUMF_K_ALL_G(128, kBf16, false, 16, 8),
    CUMF_K_ALL_G(256, kBf16, false, 32, 16),
    CUMF_K(32, kBf16, 4, true),
    CUMF_K_ALL_G(64, kBf16, true, 8, 4),
    CUMF_K_ALL_G(128, kBf16, true, 16, 8),
    CUMF_K_ALL_G(256, kBf16, true, 32, 16),
    // fp32 (rows of 4k bytes)
    CUMF_K_ALL_G(32, kFloat, false, 8, 4),
    CUMF_K_ALL_G(64, kFloat, false, 16, 8),
    CUMF_K_ALL_G(128, kFloat, false, 32, 16),
    CUMF_K_ALL_G(256, kFloat, false, 32, 16),
};

#undef CUMF_K_ALL_G
#undef CUMF_K

const KernelEntry *find_kernel(int k, int precision, int lanes) {
    const int kind = store_of_precision(precision);
    const bool sr = (precision == CUMF_BF16_SR || precision == CUMF_FP16_SR);
    const KernelEntry *first = nullptr;
    for (const KernelEntry &e : kKernels) {
        if (e.k != k || e.kind != kind || e.sr != sr) continue;
        if (lanes == 0) return &e;  // first listed = tuned default
        if (e.lanes == lanes) return &e;
        if (!first) first = &e;
    }
    return lanes == 0 ? first : nullptr;
}

}  // namespace

int default_lanes(int k, int precision) {
    const KernelEntry *e = find_kernel(k, precision, 0);
    return e ? e->lanes : 0;
}

bool lanes_supported(int k, int precision, int lanes) {
    return find_kernel(k, precision, lanes) != nullptr;
}

int workers_per_block(int lanes) { return kBlock / lanes; }

// The ring kernels need more than the default 48 KB of dynamic shared memory.
cudaError_t prepare_ring(const KernelEntry *e) {
    return cudaFuncSetAttribute(e->ring, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->ring_smem);
}

int resident_workers_of(const KernelEntry *e, bool ring, int sm_count) {
    int blocks = 0;
    if (ring) {
        if (prepare_ring(e) != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, e->ring, kBlock, e->ring_smem) != cudaSuccess)
            return 0;
    } else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, e->fn, kBlock, 0) != cudaSuccess) {
        return 0;
    }
    return blocks * sm_count * (kBlock / e->lanes);
}

int resident_workers(int k, int precision, int lanes, int sm_count) {
    const KernelEntry *e = find_kernel(k, precision, lanes);
    if (!e) return 0;
    return resident_workers_of(e, kDefaultRing != 0, sm_count);
}

// With the hot rows split into copies, or with the item rows frozen (fold-in epochs), no
// worker queues on a hot row's lines: the kernel is issue-bound while P and Q stay mostly in
// L2, and the prefetch instructions cost more than they save (c2, 480,189 x 17,770, per
// epoch: fp16 9.03 against 9.69 ms, fp32 18.2 against 19.9, bf16-SR 20.0 against 20.8; a
// 5.2M-rating fold-in epoch: fp16 0.76 against 0.85 ms, bf16-SR 1.31 against 1.37); with
// factors far beyond L2 the row loads go to DRAM and the prefetch pays again (c3, 1,000,990 x
// 624,961, 416 MB of fp16 factors: 28.2 ms with it against 31.4 without).
static int copies_prefetch(int32_t m, int32_t n, int k, int precision) {
    int dev = 0, l2 = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) {
        cudaGetLastError();
        l2 = 126 << 20;
    }
    const double bytes = ((double)m + (double)n) * k * elem_bytes(precision);
    return bytes > 2.0 * l2 ? kDefaultPrefetch : 0;
}

Tuning resolve_tuning(int k, int precision, Tuning t) {
    if (t.lanes == 0) t.lanes = default_lanes(k, precision);
    if (t.prefetch < 0) t.prefetch = kDefaultPrefetch;
    if (t.prefetch > 15) t.prefetch = 15;
    if (t.hints < 0) t.hints = kDefaultHints;
    if (t.ring < 0) t.ring = kDefaultRing;
    return t;
}

cudaError_t launch_sgd_update(const cumf_node *d_R, int64_t nnz, void *d_P, int32_t m,
                              void *d_Q, int32_t n, int k, int precision, int num_workers,
                              const Tuning &tuning, const float *d_lr, int first_epoch,
                              int n_epochs, float lambda_p, float lambda_q, uint64_t seed,
                              int *d_status, cudaStream_t stream, int *lanes_used) {
    Tuning t = resolve_tuning(k, precision, tuning);
    if (tuning.prefetch < 0 && (tuning.copies || tuning.freeze_q)) t.prefetch = copies_prefetch(m, n, k, precision);
    const KernelEntry *e = find_kernel(k, precision, t.lanes);
    if (!e) return cudaErrorInvalidValue;
    if (lanes_used) *lanes_used = e->lanes;
    if (nnz <= 0 || n_epochs <= 0 || num_workers <= 0) return cudaSuccess;
    UpdateArgs a;
    a.R = d_R;
    a.nnz = (uint64_t)nnz;
    a.P = d_P;
    a.Q = d_Q;
    a.m = (uint32_t)m;
    a.n = (uint32_t)n;
    a.lr = d_lr;
    a.first_epoch = first_epoch;
    a.n_epochs = n_epochs;
    a.num_workers = num_workers;
    a.batches = (int)batches_per_worker(nnz, num_workers);
    a.lambda_p = lambda_p;
    a.lambda_q = lambda_q;
    a.seed = seed;
    a.status = d_status;
    a.prefetch = t.prefetch;
    a.hints = t.hints;
    a.freeze_q = t.freeze_q;
    const int gpb = kBlock / e->lanes;
    const int blocks = (num_workers + gpb - 1) / gpb;
    if (t.ring) {
        cudaError_t ce = prepare_ring(e);
        if (ce != cudaSuccess) return ce;
        e->ring<<<blocks, kBlock, e->ring_smem, stream>>>(a);
    } else {
        e->fn<<<blocks, kBlock, 0, stream>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace cumf
