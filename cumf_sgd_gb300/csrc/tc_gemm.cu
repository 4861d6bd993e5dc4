// tc_gemm.cu - BF16 tensor-core GEMM for sm_103a on the 5th-generation tensor cores.
//
//   C[M x N] = act(A[M x K] * B[N x K]^T + bias[N])       (A, B bf16 row-major; fp32 accumulate)
//
// Used by the warm-start MLP (forward: activations x W^T; backward: dX = dY W and
// dW = dY^T X, given as TN products on transposed copies).  One CTA of 256 threads computes a
// 128 x BN tile (BN = 128 or 256):
//   - thread 0 is the TMA producer: operand tiles of 64 K-elements (128-byte rows) arrive by
//     cp.async.bulk.tensor.2d with the 128-byte swizzle into a ring of shared memory (2 stages
//     for K <= 1024, so two CTAs share an SM; 4 stages for longer K),
//     each stage guarded by a `full` mbarrier (armed with the expected byte count) and an
//     `empty` mbarrier;
//   - thread 32 issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=BN, K=16) four times per
//     stage, accumulating in tensor memory (BN fp32 columns from tcgen05.alloc), and
//     tcgen05.commit releases the stage to the producer through `empty`;
//   - after the last stage a commit to `done` releases the epilogue: eight warps read the
//     accumulator with tcgen05.ld (warp w: lanes 32 (w % 4).., half w / 4 of the columns, 32
//     columns at a time), add the bias, apply the activation, and pass each 32 x 32 block
//     through shared memory (the idle operand ring) so that the global stores are whole
//     128-byte lines;
//   - when the output has too few tiles to fill the GPU and K is long (the weight gradients),
//     K is split over grid.z and the partial tiles are added into a zeroed fp32 output with
//     vector atomics.
// Every mbarrier wait is bounded; on timeout the kernel records CUMF_ERR_TIMEOUT, stops
// issuing work, waits (bounded) for what it issued and releases its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "cumf_sgd.h"
#include "internal.h"

namespace cumf {

namespace {

constexpr int kTcThreads = 256;  // 8 warps: all read the accumulator in the epilogue
constexpr int kStgStride = 36;    // floats per staged row (144 bytes: 16-byte aligned, conflict-free)
constexpr int kTcBM = 128;
constexpr int kTcBK = 64;
constexpr unsigned long long kWaitNs = 2000000000ull;  // an mbarrier wait gives up after 2 s
constexpr long long kSpinLimit = 1ll << 28;            // and after this many polls in any case

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Instruction descriptor for kind::f16: D fp32 (bits 4-5 = 1), A and B bf16 (7-9, 10-12 = 1),
// both K-major (15, 16 = 0), N >> 3 at 17-22, M >> 4 at 24-28.
template <int BN>
__device__ __forceinline__ uint32_t instr_desc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of parity `parity` of an mbarrier; false after kWaitNs of global time.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const unsigned long long t0 = global_ns();
    for (long long i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 63) == 63 && global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

__device__ __forceinline__ float gelu(float x) {
    // tanh form (Hendrycks & Gimpel 2016): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
    const float c = 0.7978845608028654f;
    return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}


__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;              // leading byte offset: unused for swizzled K-major
    d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset: one 8-row atom
    d |= (uint64_t)1 << 46;              // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;              // 128-byte swizzle
    return d;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

// Epilogue of one warp's 32 rows x 32 columns (rows r0.., columns col0..; lane = row in r[]):
// the values pass through shared memory (stg, 32 x kStgStride floats) so that the global
// stores are whole 128-byte lines per 8 lanes (fp32) or 64-byte segments per 4 lanes (bf16).
// partial: fp32 partial sums added with vector atomics (split K), no bias or activation.
__device__ __forceinline__ void stage_f32(float *stg, const float (&v)[32], int lane) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q)
        *reinterpret_cast<float4 *>(stg + lane * kStgStride + 4 * q) =
            make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    __syncwarp();
}

__device__ __forceinline__ void write_f32(const float *stg, float *dst, int r0, int col0, int M, int N, int ldo,
                                          bool vec_ok, bool atomic, int lane) {
#pragma unroll
    for (int it = 0; it < 8; ++it) {
        const int row = it * 4 + (lane >> 3), c = (lane & 7) * 4;
        const int gr = r0 + row, col = col0 + c;
        if (gr >= M || col >= N) continue;
        const float4 x = *reinterpret_cast<const float4 *>(stg + row * kStgStride + c);
        float *o = dst + (size_t)gr * ldo + col;
        if (vec_ok && col + 3 < N) {
            if (atomic)
                atomicAdd(reinterpret_cast<float4 *>(o), x);
            else
                *reinterpret_cast<float4 *>(o) = x;
        } else {
            const float xs[4] = {x.x, x.y, x.z, x.w};
            for (int e = 0; e < 4 && col + e < N; ++e) {
                if (atomic)
                    atomicAdd(o + e, xs[e]);
                else
                    o[e] = xs[e];
            }
        }
    }
}

__device__ __forceinline__ void write_bf16(float *stg, const float (&v)[32], __nv_bfloat16 *dst, int r0, int col0,
                                           int M, int N, int ldo, bool vec_ok, int lane) {
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint4 w;
        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&w);
#pragma unroll
        for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(v[8 * q + 2 * e], v[8 * q + 2 * e + 1]);
        *reinterpret_cast<uint4 *>(stg + lane * kStgStride + 4 * q) = w;
    }
    __syncwarp();
#pragma unroll
    for (int it = 0; it < 4; ++it) {
        const int row = it * 8 + (lane >> 2), c = (lane & 3) * 8;
        const int gr = r0 + row, col = col0 + c;
        if (gr >= M || col >= N) continue;
        const uint4 x = *reinterpret_cast<const uint4 *>(stg + row * kStgStride + (lane & 3) * 4);
        __nv_bfloat16 *o = dst + (size_t)gr * ldo + col;
        if (vec_ok && col + 7 < N) {
            *reinterpret_cast<uint4 *>(o) = x;
        } else {
            const __nv_bfloat16 *xs = reinterpret_cast<const __nv_bfloat16 *>(&x);
            for (int e = 0; e < 8 && col + e < N; ++e) o[e] = xs[e];
        }
    }
}

__device__ __forceinline__ void epilogue_chunk(float *stg, const uint32_t (&r)[32], int r0, int col0, int M, int N,
                                               const float *__restrict__ bias, int act, void *out, int out_f32,
                                               int ldo, float *pre_out, bool partial, int lane) {
    float v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
    const bool al16 = (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
    if (partial) {
        stage_f32(stg, v, lane);
        write_f32(stg, reinterpret_cast<float *>(out), r0, col0, M, N, ldo, al16 && (ldo & 3) == 0, true, lane);
        return;
    }
    if (bias) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (col0 + j < N) v[j] += __ldg(bias + col0 + j);
    }
    if (pre_out) {
        stage_f32(stg, v, lane);
        write_f32(stg, pre_out, r0, col0, M, N, ldo,
                  (reinterpret_cast<uintptr_t>(pre_out) & 15u) == 0 && (ldo & 3) == 0, false, lane);
    }
    if (act == 1) {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = gelu(v[j]);
    }
    if (out_f32) {
        stage_f32(stg, v, lane);
        write_f32(stg, reinterpret_cast<float *>(out), r0, col0, M, N, ldo, al16 && (ldo & 3) == 0, false, lane);
    } else {
        write_bf16(stg, v, reinterpret_cast<__nv_bfloat16 *>(out), r0, col0, M, N, ldo, al16 && (ldo & 7) == 0,
                   lane);
    }
}

template <int BN, int kStages>
struct TmaSmem {
    static constexpr int A_BYTES = kTcBM * 128;  // 128 rows x 64 bf16
    static constexpr int B_BYTES = BN * 128;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int TOTAL = 1024 + kStages * STAGE + 256;  // alignment slack + barriers
};

template <int BN, int kStages>
__global__ void __launch_bounds__(kTcThreads, kStages == 2 ? 2 : 1)
tc_gemm_tma_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int M,
                   int N, int K, const float *__restrict__ bias, int act, void *out, int out_f32, int ldo,
                   float *pre_out, int *status, int splits, int no_copies) {
    using S = TmaSmem<BN, kStages>;
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;  // swizzle atoms need 1024-byte alignment
    unsigned char *bar_area = smem_raw + (base - raw) + kStages * S::STAGE;
    uint64_t *full = reinterpret_cast<uint64_t *>(bar_area);
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    int *issued_slot = abort_flag + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * BN;
    const int KT_all = (K + kTcBK - 1) / kTcBK;
    const int kt0 = (int)((long long)KT_all * blockIdx.z / splits);
    const int kt1 = (int)((long long)KT_all * (blockIdx.z + 1) / splits);
    const int KT = kt1 - kt0;

    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        *abort_flag = 0;
        *issued_slot = 0;
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 0 && KT > 0 && !no_copies) {  // TMA producer (no_copies: the wait self-test)
        for (int i = 0; i < KT; ++i) {
            const int st = i % kStages;
            if (i >= kStages && !mbar_wait(smem_u32(&empty[st]), ((i / kStages) - 1) & 1)) {
                atomicExch(abort_flag, 1);
                break;
            }
            const uint32_t fb = smem_u32(&full[st]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(S::STAGE)
                         : "memory");
            const uint32_t a_dst = base + st * S::STAGE;
            tma_load_2d(a_dst, &map_a, (kt0 + i) * kTcBK, m0, fb);
            tma_load_2d(a_dst + S::A_BYTES, &map_b, (kt0 + i) * kTcBK, n0, fb);
            *issued_slot = i + 1;
        }
    } else if (threadIdx.x == 32 && KT > 0) {  // MMA issuer
        for (int i = 0; i < KT; ++i) {
            const int st = i % kStages;
            if (!mbar_wait(smem_u32(&full[st]), (i / kStages) & 1)) {
                atomicExch(abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t a0 = base + st * S::STAGE, b0 = a0 + S::A_BYTES;
#pragma unroll
            for (int s = 0; s < kTcBK / 16; ++s) {
                const uint32_t acc = (i > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(sw128_desc(a0 + s * 32)), "l"(sw128_desc(b0 + s * 32)), "r"(instr_desc<BN>()), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&empty[st]))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         smem_u32(done))
                     : "memory");
    }
    // Everyone waits for the accumulator (bounded), then agrees on whether it is valid.
    int ok = 1;
    if (KT > 0) ok = mbar_wait(smem_u32(done), 0) ? 1 : 0;
    __syncwarp();
    ok = __syncthreads_and(ok && (*abort_flag == 0));
    if (!ok) {
        if (threadIdx.x == 0) {
            if (status) atomicExch(status, (int)CUMF_ERR_TIMEOUT);
            // Bounded drain: the last copy issued into each stage, then every MMA.
            const int issued = *issued_slot;
            for (int st = 0; st < kStages && st < issued; ++st) {
                const int last = st + ((issued - 1 - st) / kStages) * kStages;
                mbar_wait(smem_u32(&full[st]), (last / kStages) & 1);
            }
            mbar_wait(smem_u32(done), 0);
        }
    } else if (KT > 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // Warp w reads tensor-memory lanes 32 (w % 4).. (its rows) and half w / 4 of the
        // columns.  The operand ring is idle now and holds each warp's staging block.
        float *stg = reinterpret_cast<float *>(smem_raw + (base - raw)) + warp * (32 * kStgStride);
        const int quarter = warp & 3, half = warp >> 2;
        const int r0 = m0 + quarter * 32;
        for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2) && n0 + c0 < N; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                "[%32];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            epilogue_chunk(stg, r, r0, n0 + c0, M, N, bias, act, out, out_f32, ldo, pre_out, splits > 1, lane);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
    }
}

// ---- persistent variant (many output tiles, no split K) ----------------------------------
//
// One CTA per SM walks tiles t = blockIdx.x, blockIdx.x + gridDim.x, ... (the two n-tiles of an
// m-block are adjacent, so their A rows are read once from DRAM).  Warp 0 (one lane) streams
// operand stages through the ring across tile boundaries; warp 1 (one lane) issues the MMAs
// into one of two tensor-memory accumulators (tile j uses accumulator j % 2) and commits
// `tfull`; warps 2-5 drain an accumulator (tcgen05.ld, bias, activation, staged coalesced
// stores) and release it through `tempty` while the next tile's MMAs fill the other one.
constexpr int kPersThreads = 192;

template <int BN, int kStages>
struct PersSmem {
    static constexpr int A_BYTES = kTcBM * 128;
    static constexpr int B_BYTES = BN * 128;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int STG = 4 * 32 * kStgStride * 4;  // four epilogue warps' staging blocks
    static constexpr int TOTAL = 1024 + kStages * STAGE + STG + 256;
};

__device__ __forceinline__ bool aborted(const int *flag) { return *reinterpret_cast<const volatile int *>(flag) != 0; }

template <int BN, int kStages>
__global__ void __launch_bounds__(kPersThreads, 1)
tc_gemm_persistent_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int M,
                          int N, int K, const float *__restrict__ bias, int act, void *out, int out_f32, int ldo,
                          float *pre_out, int *status) {
    using S = PersSmem<BN, kStages>;
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;  // swizzle atoms need 1024-byte alignment
    unsigned char *aligned = smem_raw + (base - raw);
    float *stg_all = reinterpret_cast<float *>(aligned + kStages * S::STAGE);
    uint64_t *full = reinterpret_cast<uint64_t *>(aligned + kStages * S::STAGE + S::STG);
    uint64_t *empty = full + kStages;
    uint64_t *tfull = empty + kStages;
    uint64_t *tempty = tfull + 2;
    uint64_t *mma_done = tempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    int *issued_slot = abort_flag + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_n = (N + BN - 1) / BN;
    const int tiles = ((M + kTcBM - 1) / kTcBM) * tiles_n;
    const int my_tiles = (int)blockIdx.x < tiles ? (tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    const int KT = (K + kTcBK - 1) / kTcBK;

    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[i])));
        }
        for (int i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&tfull[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(smem_u32(&tempty[i])));  // one per epilogue warp
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mma_done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        *abort_flag = 0;
        *issued_slot = 0;
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // TMA producer
            int it = 0;
            for (int j = 0; j < my_tiles && !aborted(abort_flag); ++j) {
                const int t = (int)blockIdx.x + j * (int)gridDim.x;
                const int tm = t / tiles_n, tn = t % tiles_n;
                for (int kk = 0; kk < KT; ++kk, ++it) {
                    const int st = it % kStages;
                    if (it >= kStages && !mbar_wait(smem_u32(&empty[st]), ((it / kStages) - 1) & 1)) {
                        atomicExch(abort_flag, 1);
                        break;
                    }
                    const uint32_t fb = smem_u32(&full[st]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(S::STAGE)
                                 : "memory");
                    const uint32_t a_dst = base + st * S::STAGE;
                    tma_load_2d(a_dst, &map_a, kk * kTcBK, tm * kTcBM, fb);
                    tma_load_2d(a_dst + S::A_BYTES, &map_b, kk * kTcBK, tn * BN, fb);
                    *issued_slot = it + 1;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            int it = 0;
            bool ok = true;
            for (int j = 0; j < my_tiles && ok; ++j) {
                const int acc = j & 1;
                if (j >= 2 && !mbar_wait(smem_u32(&tempty[acc]), ((j >> 1) - 1) & 1)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(acc * BN);
                for (int kk = 0; kk < KT; ++kk, ++it) {
                    const int st = it % kStages;
                    if (!mbar_wait(smem_u32(&full[st]), (it / kStages) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t a0 = base + st * S::STAGE, b0 = a0 + S::A_BYTES;
#pragma unroll
                    for (int sub = 0; sub < kTcBK / 16; ++sub) {
                        const uint32_t accum = (kk > 0 || sub > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                            "l"(sw128_desc(a0 + sub * 32)), "l"(sw128_desc(b0 + sub * 32)), "r"(instr_desc<BN>()),
                            "r"(accum));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     smem_u32(&empty[st]))
                                 : "memory");
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smem_u32(&tfull[acc]))
                             : "memory");
            }
            if (!ok) atomicExch(abort_flag, 1);
            // Tracks every MMA issued above: the accumulators may be freed once it completes.
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(mma_done))
                         : "memory");
        }
    } else {  // epilogue warps 2-5: tensor-memory lanes 32 (warp % 4)..
        const int quarter = warp & 3;
        float *stg = stg_all + (warp - 2) * (32 * kStgStride);
        for (int j = 0; j < my_tiles; ++j) {
            const int acc = j & 1;
            const int t = (int)blockIdx.x + j * (int)gridDim.x;
            const int tm = t / tiles_n, tn = t % tiles_n;
            int ok = mbar_wait(smem_u32(&tfull[acc]), (j >> 1) & 1) ? 1 : 0;
            ok = __all_sync(0xffffffffu, ok) && !aborted(abort_flag);
            if (!ok) {
                if (lane == 0) atomicExch(abort_flag, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int r0 = tm * kTcBM + quarter * 32, n0 = tn * BN;
            for (int c0 = 0; c0 < BN && n0 + c0 < N; c0 += 32) {
                uint32_t r[32];
                const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * BN + c0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                    "[%32];\n"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                      "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                      "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                epilogue_chunk(stg, r, r0, n0 + c0, M, N, bias, act, out, out_f32, ldo, pre_out, false, lane);
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&tempty[acc])) : "memory");
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // Bounded drain: every MMA, then (after an abort) the last copy issued into each stage.
        mbar_wait(smem_u32(mma_done), 0);
        if (aborted(abort_flag)) {
            if (status) atomicExch(status, (int)CUMF_ERR_TIMEOUT);
            const int issued = *issued_slot;
            for (int st = 0; st < kStages && st < issued; ++st) {
                const int last = st + ((issued - 1 - st) / kStages) * kStages;
                mbar_wait(smem_u32(&full[st]), (last / kStages) & 1);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * BN));
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    }
    return fn;
}

// rows x K bf16 row-major operand, tiles of box_rows x 64 with 128-byte swizzle.
bool make_map(CUtensorMap *map, const void *ptr, int rows, int K, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

template <int BN, int ST>
cudaError_t launch_variant(dim3 grid, const CUtensorMap &ma, const CUtensorMap &mb, int M, int N, int K,
                           const float *bias, int act, void *out, int out_f32, int ldo, float *pre_out, int *status,
                           int splits, cudaStream_t s, int no_copies = 0) {
    const int sm = TmaSmem<BN, ST>::TOTAL;
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_tma_kernel<BN, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    tc_gemm_tma_kernel<BN, ST><<<grid, kTcThreads, sm, s>>>(ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out,
                                                            status, splits, no_copies);
    return cudaGetLastError();
}

template <int BN, int ST>
cudaError_t launch_persistent(int grid, const CUtensorMap &ma, const CUtensorMap &mb, int M, int N, int K,
                              const float *bias, int act, void *out, int out_f32, int ldo, float *pre_out, int *status,
                              cudaStream_t s) {
    const int sm = PersSmem<BN, ST>::TOTAL;
    cudaError_t e =
        cudaFuncSetAttribute(tc_gemm_persistent_kernel<BN, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    tc_gemm_persistent_kernel<BN, ST><<<grid, kPersThreads, sm, s>>>(ma, mb, M, N, K, bias, act, out, out_f32, ldo,
                                                                     pre_out, status);
    return cudaGetLastError();
}

int sm_count_of_current_device() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms;
}

cudaError_t launch_tc_gemm(const void *A, const void *B, int M, int N, int K, const float *bias, int act,
                           void *out, int out_f32, int ldo, float *pre_out, int *status, cudaStream_t s) {
    if (M <= 0 || N <= 0 || K <= 0 || (K % 8) != 0) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15)) return cudaErrorInvalidValue;
    const int sms = sm_count_of_current_device();
    const int nsm = sms > 0 ? sms : 152;
    const int tiles_m = (M + kTcBM - 1) / kTcBM;
    const int kt = (K + kTcBK - 1) / kTcBK;
    // Short K (at most 16 stages of 64): a 2-stage ring, so two CTAs share an SM and
    // one CTA's epilogue overlaps another's loads.  Long K: a 4-stage ring, one CTA per SM.
    const bool short_k = kt <= 16;
    // Split K when the output has too few tiles to fill the GPU and K is long (weight
    // gradients): about one wave of CTAs, each with at least 8 stages.
    const bool plain = out_f32 && !bias && act == 0 && !pre_out;
    auto splits_for = [&](long long tiles) -> int {
        if (!plain || short_k || tiles >= nsm) return 1;
        return (int)std::max(1ll, std::min<long long>(kt / 8, nsm / tiles));
    };
    // 128 x 256 tiles (one A tile feeds twice the columns) unless they leave most of a wave
    // idle: 128 x 128 tiles when those give at least 1.5 times the CTAs and the wide ones do not
    // fill the SMs (the MLP's 4096-row batches: 64 wide tiles, or weight gradients whose split
    // is capped by K).
    bool wide = N > 128;
    if (wide) {
        const long long tw = (long long)tiles_m * ((N + 255) / 256), tn = (long long)tiles_m * ((N + 127) / 128);
        const long long cw = tw * splits_for(tw), cn = tn * splits_for(tn);
        wide = cw >= nsm || 2 * cn < 3 * cw;
    }
    const int BN = wide ? 256 : 128;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, kTcBM) || !make_map(&mb, B, N, K, BN)) return cudaErrorInvalidValue;
    const int tiles_n = (N + BN - 1) / BN;
    const int splits = splits_for((long long)tiles_m * tiles_n);
    if (splits > 1) {
        cudaError_t e = cudaMemset2DAsync(out, (size_t)ldo * 4, 0, (size_t)N * 4, M, s);
        if (e != cudaSuccess) return e;
    }
    // Enough output tiles for two per SM: the persistent kernel, whose epilogues overlap the
    // next tiles' loads and MMAs.
    if (splits == 1 && sms > 0 && (long long)tiles_m * tiles_n >= 2ll * sms) {
        const int g = std::min(tiles_m * tiles_n, sms);
        return wide ? launch_persistent<256, 4>(g, ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out, status, s)
                    : launch_persistent<128, 6>(g, ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out, status, s);
    }
    const dim3 grid(tiles_m, tiles_n, splits);
    if (wide)
        return short_k ? launch_variant<256, 2>(grid, ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out, status,
                                                splits, s)
                       : launch_variant<256, 4>(grid, ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out, status,
                                                splits, s);
    return short_k ? launch_variant<128, 2>(grid, ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out, status,
                                            splits, s)
                   : launch_variant<128, 4>(grid, ma, mb, M, N, K, bias, act, out, out_f32, ldo, pre_out, status,
                                            splits, s);
}

}  // namespace cumf

using namespace cumf;

extern "C" int cumf_tc_gemm(const void *d_A, const void *d_B, int M, int N, int K, const float *d_bias, int act,
                            void *d_out, int out_f32, int ldo, float *d_pre, int *d_status, void *stream) {
    if (!d_A || !d_B || !d_out || M <= 0 || N <= 0 || K <= 0 || (K % 8) != 0 || ldo < N)
        return fail(CUMF_ERR_ARG, "tc_gemm: bad arguments (K must be a multiple of 8, ldo >= N)");
    if (act != 0 && act != 1) return fail(CUMF_ERR_ARG, "tc_gemm: act must be 0 (identity) or 1 (gelu)");
    CUMF_CUDA(launch_tc_gemm(d_A, d_B, M, N, K, d_bias, act, d_out, out_f32, ldo, d_pre, d_status,
                             (cudaStream_t)stream));
    return CUMF_OK;
}

extern "C" int cumf_selftest_wait_timeout(int *status_out, double *seconds) {
    if (!status_out) return fail(CUMF_ERR_ARG, "selftest: status_out is NULL");
    *status_out = 0;
    // One 128 x 128 x 64 tile whose producer issues no copies: the MMA thread's wait on the
    // stage barrier runs out, the kernel records CUMF_ERR_TIMEOUT, drains and frees its tensor
    // memory; then an ordinary product on the same context must still be right.
    const int M = 128, N = 128, K = 64;
    void *buf = nullptr;
    const size_t ab = (size_t)M * K * 2, bb = (size_t)N * K * 2, ob = (size_t)M * N * 4;
    CUMF_CUDA(cudaMalloc(&buf, ab + bb + ob + 16));
    char *A = static_cast<char *>(buf);
    char *B = A + ab;
    float *O = reinterpret_cast<float *>(B + bb);
    int *st = reinterpret_cast<int *>(reinterpret_cast<char *>(O) + ob);
    int rc = CUMF_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    do {
        cudaError_t e = cudaMemset(buf, 0, ab + bb + ob + 16);
        if (e == cudaSuccess) {  // A = B = bf16 1.0: every output element is K
            std::vector<uint16_t> ones((M > N ? M : N) * K, 0x3f80);
            e = cudaMemcpy(A, ones.data(), ab, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(B, ones.data(), bb, cudaMemcpyHostToDevice);
        }
        CUtensorMap ma, mb;
        if (e == cudaSuccess && (!make_map(&ma, A, M, K, kTcBM) || !make_map(&mb, B, N, K, 128))) {
            rc = fail(CUMF_ERR_CUDA, "selftest: tensor maps");
            break;
        }
        if (e == cudaSuccess) e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
        if (e == cudaSuccess)
            e = launch_variant<128, 2>(dim3(1, 1, 1), ma, mb, M, N, K, nullptr, 0, O, 1, N, nullptr, st, 1, 0, 1);
        if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess) e = cudaMemcpy(status_out, st, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "selftest: timed-out launch");
            break;
        }
        if (seconds) *seconds = ms * 1e-3;
        // The context is usable: an ordinary product gives K everywhere.
        e = launch_tc_gemm(A, B, M, N, K, nullptr, 0, O, 1, N, nullptr, nullptr, 0);
        std::vector<float> host((size_t)M * N, 0.f);
        if (e == cudaSuccess) e = cudaMemcpy(host.data(), O, ob, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "selftest: product after the timeout");
            break;
        }
        for (float v : host)
            if (v != (float)K) {
                rc = fail(CUMF_ERR_CUDA, "selftest: product after the timeout is wrong");
                break;
            }
    } while (0);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    return rc;
}
