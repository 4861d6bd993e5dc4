// tc_gemm.cu - BF16 tensor-core GEMM for sm_103a on the 5th-generation tensor cores.
//
//   C[M x N] = act(A[M x K] * B[N x K]^T + bias[N])       (A, B bf16 row-major; fp32 accumulate)
//
// Used by the warm-start MLP (forward: activations x W^T; backward: dX = dY W and
// dW = dY^T X, given as TN products on transposed copies).  One CTA of 128 threads computes a
// 128 x BN tile:
//   - operand tiles of 64 K-elements are copied with cp.async into shared memory in the
//     tcgen05 no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix; the
//     K-adjacent core matrix at +128 bytes, the next 8 rows at +1024 bytes), two stages;
//   - one elected thread issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=BN, K=16) four
//     times per stage, accumulating in tensor memory (BN fp32 columns allocated with
//     tcgen05.alloc), and tcgen05.commit arrives on an mbarrier per stage;
//   - the epilogue reads the accumulator with tcgen05.ld (32 lanes x 32 columns per warp),
//     adds the bias, applies the activation and stores bf16 or fp32.
// Every mbarrier wait is bounded; on timeout the kernel records CUMF_ERR_TIMEOUT, stops
// issuing work, waits (bounded) for what it issued and releases its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cumf_sgd.h"
#include "internal.h"

namespace cumf {

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcBM = 128;
constexpr int kTcBK = 64;
constexpr long long kSpinLimit = 1ll << 24;  // try_wait polls before giving up (seconds)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset >> 4
// (16-29), stride byte offset >> 4 (32-45), descriptor version 1 (46-47), base offset 0,
// relative LBO mode, no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t mat_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor for kind::f16: D fp32 (bits 4-5 = 1), A and B bf16 (7-9, 10-12 = 1),
// both K-major (15, 16 = 0), N >> 3 at 17-22, M >> 4 at 24-28.
template <int BN>
__device__ __forceinline__ uint32_t instr_desc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
}

__device__ __forceinline__ void cp16(uint32_t dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long long i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ float gelu(float x) {
    // tanh form (Hendrycks & Gimpel 2016): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
    const float c = 0.7978845608028654f;
    return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}

// Copies a rows x 64 bf16 tile (rows from r0, K from k0) into the core-matrix layout.
// Out-of-range rows are zero-filled.
template <int ROWS>
__device__ __forceinline__ void load_tile(uint32_t sdst, const __nv_bfloat16 *G, int nrows, int K, int r0, int k0) {
    constexpr int CHUNKS = ROWS * (kTcBK / 8);
#pragma unroll 4
    for (int c = threadIdx.x; c < CHUNKS; c += kTcThreads) {
        const int row = c >> 3, kc = c & 7;
        const int gr = r0 + row;
        const bool ok = gr < nrows;
        const __nv_bfloat16 *src = G + (size_t)(ok ? gr : 0) * K + k0 + kc * 8;
        const uint32_t dst = sdst + (uint32_t)(((row >> 3) * 8 + kc) * 128 + (row & 7) * 16);
        cp16(dst, src, ok ? 16u : 0u);
    }
}

template <int BN>
struct TcSmem {
    static constexpr int A_BYTES = kTcBM * kTcBK * 2;
    static constexpr int B_BYTES = BN * kTcBK * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int TOTAL = 2 * STAGE + 64;  // + mbarriers and the TMEM address
};

template <int BN>
__global__ void __launch_bounds__(kTcThreads, 1)
tc_gemm_kernel(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B, int M, int N, int K,
               const float *__restrict__ bias, int act, void *out, int out_f32, int ldo, float *pre_out,
               int *status) {
    using S = TcSmem<BN>;
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t sbase = smem_u32(smem);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + 2 * S::STAGE);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 2 * S::STAGE + 32);
    const uint32_t mbar0 = smem_u32(&mbar[0]), mbar1 = smem_u32(&mbar[1]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * BN;

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar1));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
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

    const int KT = K / kTcBK;
    bool alive = true;
    // stage 0 <- k-tile 0
    load_tile<kTcBM>(sbase, A, M, K, m0, 0);
    load_tile<BN>(sbase + S::A_BYTES, B, N, K, n0, 0);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    for (int kt = 0; kt < KT && alive; ++kt) {
        const int st = kt & 1;
        if (kt + 1 < KT) {
            if (kt >= 1) {  // stage st^1 was read by the MMAs of k-tile kt-1
                const int timed_out = !mbar_wait(st ? mbar0 : mbar1, ((kt - 1) >> 1) & 1);
                if (__syncthreads_or(timed_out)) {  // every thread takes the same branch
                    alive = false;
                    break;
                }
            }
            const uint32_t nb = sbase + (st ^ 1) * S::STAGE;
            load_tile<kTcBM>(nb, A, M, K, m0, (kt + 1) * kTcBK);
            load_tile<BN>(nb + S::A_BYTES, B, N, K, n0, (kt + 1) * kTcBK);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // cp.async writes -> tensor core reads
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t a0 = sbase + st * S::STAGE, b0 = a0 + S::A_BYTES;
#pragma unroll
            for (int s = 0; s < kTcBK / 16; ++s) {
                const uint64_t ad = mat_desc(a0 + s * 256, 128, 1024);
                const uint64_t bd = mat_desc(b0 + s * 256, 128, 1024);
                const uint32_t acc = (kt > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(instr_desc<BN>()), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             st ? mbar1 : mbar0)
                         : "memory");
        }
    }
    // The last commit covers every MMA issued before it.
    bool done = false;
    if (alive && KT > 0) {
        const int last = KT - 1;
        done = __syncthreads_and(mbar_wait((last & 1) ? mbar1 : mbar0, (last >> 1) & 1));
    }
    if (!done || !alive) {
        if (threadIdx.x == 0 && status) atomicExch(status, (int)CUMF_ERR_TIMEOUT);
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        // Bounded drain of anything still in flight on either stage before the memory is freed.
        mbar_wait(mbar0, 0);
        mbar_wait(mbar1, 0);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < BN; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
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
            if (row < M) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int col = n0 + c0 + j;
                    if (col < N) {
                        float v = __uint_as_float(r[j]) + (bias ? bias[col] : 0.f);
                        if (pre_out) pre_out[(size_t)row * ldo + col] = v;
                        if (act == 1) v = gelu(v);
                        if (out_f32)
                            reinterpret_cast<float *>(out)[(size_t)row * ldo + col] = v;
                        else
                            reinterpret_cast<__nv_bfloat16 *>(out)[(size_t)row * ldo + col] = __float2bfloat16_rn(v);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
    }
}

}  // namespace

cudaError_t launch_tc_gemm(const void *A, const void *B, int M, int N, int K, const float *bias, int act,
                           void *out, int out_f32, int ldo, float *pre_out, int *status, cudaStream_t s) {
    if (M <= 0 || N <= 0 || K <= 0 || (K % kTcBK) != 0) return cudaErrorInvalidValue;
    const bool wide = N > 128;
    const dim3 grid((M + kTcBM - 1) / kTcBM, (N + (wide ? 256 : 128) - 1) / (wide ? 256 : 128));
    if (wide) {
        const int sm = TcSmem<256>::TOTAL;
        cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (e != cudaSuccess) return e;
        tc_gemm_kernel<256><<<grid, kTcThreads, sm, s>>>(reinterpret_cast<const __nv_bfloat16 *>(A),
                                                         reinterpret_cast<const __nv_bfloat16 *>(B), M, N, K, bias,
                                                         act, out, out_f32, ldo, pre_out, status);
    } else {
        const int sm = TcSmem<128>::TOTAL;
        cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (e != cudaSuccess) return e;
        tc_gemm_kernel<128><<<grid, kTcThreads, sm, s>>>(reinterpret_cast<const __nv_bfloat16 *>(A),
                                                         reinterpret_cast<const __nv_bfloat16 *>(B), M, N, K, bias,
                                                         act, out, out_f32, ldo, pre_out, status);
    }
    return cudaGetLastError();
}

}  // namespace cumf

using namespace cumf;

extern "C" int cumf_tc_gemm(const void *d_A, const void *d_B, int M, int N, int K, const float *d_bias, int act,
                            void *d_out, int out_f32, int ldo, float *d_pre, int *d_status, void *stream) {
    if (!d_A || !d_B || !d_out || M <= 0 || N <= 0 || K <= 0 || (K % 64) != 0 || ldo < N)
        return fail(CUMF_ERR_ARG, "tc_gemm: bad arguments (K must be a multiple of 64, ldo >= N)");
    if (act != 0 && act != 1) return fail(CUMF_ERR_ARG, "tc_gemm: act must be 0 (identity) or 1 (gelu)");
    CUMF_CUDA(launch_tc_gemm(d_A, d_B, M, N, K, d_bias, act, d_out, out_f32, ldo, d_pre, d_status,
                             (cudaStream_t)stream));
    return CUMF_OK;
}
