// device_common.cuh - storage traits and small device helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "cumf_sgd.h"
#include "rng.h"

namespace cumf {

// Storage class of a factor matrix.  The arithmetic is always fp32 (the reference converts
// half -> float, updates in float and stores with __float2half, warp32.h:62-99).
enum StoreKind { kHalf = 0, kBf16 = 1, kFloat = 2 };

__host__ __device__ constexpr int store_bytes(int kind) { return kind == kFloat ? 4 : 2; }

__host__ __device__ constexpr int store_of_precision(int precision) {
    return (precision == CUMF_FP16 || precision == CUMF_FP16_SR) ? kHalf
         : (precision == CUMF_BF16 || precision == CUMF_BF16_SR) ? kBf16
         : kFloat;
}

// ---- 16-byte words of a factor row <-> fp32 pairs ----------------------------------
// A lane owns E consecutive elements of a row, moved as E*bytes/16 uint4 words.  The kernel
// walks a word as kPairs element pairs, widening a pair to fp32 only while it is in use, so
// few registers stay live per record.
template <int KIND>
struct Conv;

// Stochastic rounding of x to a neighbouring half: up with probability equal to the
// distance from the lower neighbour over the gap.  u is uniform on [0,1).
__device__ __forceinline__ __half half_round_sr(float x, float u) {
    const __half lo = __float2half_rd(x);
    const __half hi = __float2half_ru(x);
    const float flo = __half2float(lo), fhi = __half2float(hi);
    return (x - flo > u * (fhi - flo)) ? hi : lo;
}

// bf16 stochastic rounding: add 16 random bits below the kept mantissa, then truncate.
__device__ __forceinline__ uint32_t bf16_round_sr(float x, uint32_t r16) {
    const uint32_t b = __float_as_uint(x);
    if ((b & 0x7f800000u) == 0x7f800000u)  // inf / nan: round to nearest
        return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
    return (b + r16) >> 16;
}

template <>
struct Conv<kHalf> {
    static constexpr int kPairs = 4;  // element pairs per 16-byte word
    __device__ __forceinline__ static float2 get(const uint4 &w, int h) {
        const uint32_t x = (&w.x)[h];
        return __half22float2(*reinterpret_cast<const __half2 *>(&x));
    }
    __device__ __forceinline__ static void put(uint4 &w, int h, float a, float b) {
        __half2 t = __floats2half2_rn(a, b);
        (&w.x)[h] = *reinterpret_cast<uint32_t *>(&t);
    }
    __device__ __forceinline__ static void put_sr(uint4 &w, int h, float a, float b, uint32_t bits) {
        const __half lo = half_round_sr(a, (float)(bits & 0xffffu) * (1.0f / 65536.0f));
        const __half hi = half_round_sr(b, (float)(bits >> 16) * (1.0f / 65536.0f));
        (&w.x)[h] = (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
    }
};

template <>
struct Conv<kBf16> {
    static constexpr int kPairs = 4;
    __device__ __forceinline__ static float2 get(const uint4 &w, int h) {
        const uint32_t x = (&w.x)[h];
        return make_float2(__uint_as_float(x << 16), __uint_as_float(x & 0xffff0000u));
    }
    __device__ __forceinline__ static void put(uint4 &w, int h, float a, float b) {
        __nv_bfloat162 t = __floats2bfloat162_rn(a, b);
        (&w.x)[h] = *reinterpret_cast<uint32_t *>(&t);
    }
    __device__ __forceinline__ static void put_sr(uint4 &w, int h, float a, float b, uint32_t bits) {
        (&w.x)[h] = (bf16_round_sr(a, bits & 0xffffu) & 0xffffu) | (bf16_round_sr(b, bits >> 16) << 16);
    }
};

template <>
struct Conv<kFloat> {
    static constexpr int kPairs = 2;
    __device__ __forceinline__ static float2 get(const uint4 &w, int h) {
        return make_float2(__uint_as_float((&w.x)[2 * h]), __uint_as_float((&w.x)[2 * h + 1]));
    }
    __device__ __forceinline__ static void put(uint4 &w, int h, float a, float b) {
        (&w.x)[2 * h] = __float_as_uint(a);
        (&w.x)[2 * h + 1] = __float_as_uint(b);
    }
    __device__ __forceinline__ static void put_sr(uint4 &w, int h, float a, float b, uint32_t) {
        put(w, h, a, b);
    }
};

// Single-element conversions (init, export).
template <int KIND>
struct Scalar;
template <>
struct Scalar<kHalf> {
    using T = __half;
    __device__ __forceinline__ static T from_float(float x) { return __float2half_rn(x); }
    __device__ __forceinline__ static float to_float(T x) { return __half2float(x); }
};
template <>
struct Scalar<kBf16> {
    using T = __nv_bfloat16;
    __device__ __forceinline__ static T from_float(float x) { return __float2bfloat16_rn(x); }
    __device__ __forceinline__ static float to_float(T x) { return __bfloat162float(x); }
};
template <>
struct Scalar<kFloat> {
    using T = float;
    __device__ __forceinline__ static T from_float(float x) { return x; }
    __device__ __forceinline__ static float to_float(T x) { return x; }
};

// Cache-hinted 16-byte accesses.  Factor rows are read through L2 only (ld.global.cg):
// other SMs write them concurrently (Hogwild), and a stale L1 copy would hide those writes.
// `pol` is an L2 cache policy from createpolicy (evict_last keeps the factor working set
// resident while the ratings stream past with evict_first).
__device__ __forceinline__ uint4 ld_row(const uint4 *p) { return __ldcg(p); }
__device__ __forceinline__ void st_row(uint4 *p, uint4 v) { __stcg(p, v); }

__device__ __forceinline__ uint64_t l2_policy(bool hint, bool keep) {
    uint64_t pol;
    if (!hint)
        asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;\n" : "=l"(pol));
    else if (keep)
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(pol));
    else
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ uint4 ld_row_hint(const uint4 *p, uint64_t pol) {
    uint4 v;
    asm volatile("ld.global.cg.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;\n"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_row_hint(uint4 *p, uint4 v, uint64_t pol) {
    asm volatile("st.global.cg.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;\n" ::"l"(p), "r"(v.x),
                 "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2::evict_last [%0];\n" ::"l"(p));
}

}  // namespace cumf
