// text_parse.cu - rating text -> 12-byte records on the GPU.
//
// Replaces data/netflix/transform.cpp:9-47, which skips three header lines with
// fscanf("%[^\n]\n") (transform.cpp:31-33) and then reads whitespace-separated triples with
// fscanf("%d %d %f") until the first failure, writing {int u, int v, float r} per triple
// (transform.cpp:36-42).
//
// GPU layout: the text sits in HBM; each thread owns a 64-byte segment.
//   1. count_tokens_kernel: a token starts at a non-space byte whose predecessor is a space
//      (or the start of the data).  Per-thread start masks are popcounted and reduced per
//      block (256 threads = 16 KB of text).
//   2. scan_blocks_kernel: exclusive scan of the block counts (one block) and the total.
//   3. parse_tokens_kernel: the same masks, a block-wide scan of the thread counts gives
//      every token its global index t; token t is field t % 3 of record t / 3 and is parsed
//      by the thread that owns its first byte (u, v as %d; r as %f) and stored in place.
// Decimal to float conversion is correctly rounded (the result strtof gives):
//   - w <= 2^24 and |q| <= 10 (w = significand digits, q = decimal exponent): one IEEE
//     float multiply or divide of exact operands (Clinger's fast path);
//   - w < 2^53 and |q| <= 22: one IEEE double operation, exact unless the double lands on a
//     midpoint between two floats (checked);
//   - otherwise the double approximation names a candidate within one float ulp and the
//     candidate's two midpoints are compared exactly with w * 10^q in 512-bit integers.
// Strictness (differences from fscanf, which stops silently or writes stale fields): a
// malformed token, an id outside int32, a rating needing more than 19 significant digits to
// round, or a token count that is not a multiple of 3 is an error (CUMF_ERR_FORMAT) naming
// the byte offset.  Hexadecimal floats and nan(...) payloads are rejected.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <vector>
#include <string>

#include "cumf_sgd.h"
#include "internal.h"
#include "text_token.h"

namespace cumf {

namespace {

constexpr int kSeg = 64;                         // bytes per thread
constexpr int kTB = 256;                         // threads per block
constexpr int64_t kBlockBytes = (int64_t)kSeg * kTB;
constexpr int kStage = (int)kBlockBytes + 64;   // a block's text plus the halo staged by the parse
constexpr int kScanThreads = 1024;
constexpr int kMaxToken = 1024;                  // longer tokens are rejected

enum : uint32_t { kBadInt = 1, kBadIntRange = 2, kBadFloat = 3, kBadDigits = 4, kBadLong = 5 };

__device__ __forceinline__ bool is_space(uint32_t c) { return c == 32u || (c - 9u) <= 4u; }

// Bit j: byte j of the 16 is not a space.
__device__ __forceinline__ uint64_t nonspace16(uint4 v) {
    const uint64_t lo = ((uint64_t)v.y << 32) | v.x, hi = ((uint64_t)v.w << 32) | v.z;
    return (uint64_t)(~(text_token::byte_flags(text_token::space_bytes(lo)) |
                        (text_token::byte_flags(text_token::space_bytes(hi)) << 8)) & 0xffffu);
}

// Bit j of the result: byte seg+j is inside [start, len) and is not a space.
__device__ __forceinline__ uint64_t nonspace_mask(const unsigned char *__restrict__ t, int64_t seg, int64_t start,
                                                  int64_t len) {
    uint64_t ns = 0;
    if (seg + kSeg <= len) {
        const uint4 *p = reinterpret_cast<const uint4 *>(t + seg);
#pragma unroll
        for (int w = 0; w < 4; ++w) ns |= nonspace16(__ldg(p + w)) << (16 * w);
    } else {
        for (int j = 0; j < kSeg && seg + j < len; ++j)
            if (!is_space(__ldg(t + seg + j))) ns |= 1ull << j;
    }
    if (start > seg) ns &= (start - seg >= kSeg) ? 0ull : (~0ull << (start - seg));
    return ns;
}

// Token starts within the segment (a bit per byte).
__device__ __forceinline__ uint64_t start_mask(const unsigned char *__restrict__ t, int64_t seg, int64_t start,
                                               int64_t len) {
    if (seg >= len || seg + kSeg <= start) return 0;
    const uint64_t ns = nonspace_mask(t, seg, start, len);
    const uint64_t prev = (seg - 1 >= start && !is_space(__ldg(t + seg - 1))) ? 1ull : 0ull;
    return ns & ~((ns << 1) | prev);
}

__global__ void __launch_bounds__(kTB) count_tokens_kernel(const unsigned char *__restrict__ t, int64_t start,
                                                           int64_t len, unsigned long long *block_counts) {
    const int64_t seg = ((int64_t)blockIdx.x * kTB + threadIdx.x) * kSeg;
    unsigned long long c = (unsigned long long)__popcll(start_mask(t, seg, start, len));
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ unsigned long long s_w[kTB / 32];
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < kTB / 32; ++w) s += s_w[w];
        block_counts[blockIdx.x] = s;
    }
}

// In place: counts[b] <- sum of counts[0..b); counts[nb] <- total.
__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(unsigned long long *counts, int64_t nb) {
    const int64_t per = (nb + kScanThreads - 1) / kScanThreads;
    const int64_t a = threadIdx.x * per, b = min(nb, a + per);
    unsigned long long s = 0;
    for (int64_t i = a; i < b; ++i) s += counts[i];
    __shared__ unsigned long long s_part[kScanThreads];
    s_part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {  // Hillis-Steele inclusive scan
        const unsigned long long x = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0ull;
        __syncthreads();
        s_part[threadIdx.x] += x;
        __syncthreads();
    }
    unsigned long long run = s_part[threadIdx.x] - s;  // exclusive
    for (int64_t i = a; i < b; ++i) {
        const unsigned long long c = counts[i];
        counts[i] = run;
        run += c;
    }
    if (threadIdx.x == kScanThreads - 1) counts[nb] = s_part[kScanThreads - 1];
}

// ---- exact decimal -> float ---------------------------------------------------------------

__device__ __forceinline__ float pow10f_exact(int e) {  // 10^e, e in [0, 10]: exact floats
    float p = 1.f;
    for (int i = 0; i < e; ++i) p *= 10.f;
    return p;
}
__device__ __forceinline__ double pow10d_exact(int e) {  // 10^e, e in [0, 22]: exact doubles
    double p = 1.0;
    for (int i = 0; i < e; ++i) p *= 10.0;
    return p;
}

struct Big {
    uint32_t l[16];  // little-endian 32-bit limbs, 512 bits
};
__device__ __forceinline__ void big_set(Big &b, uint64_t v) {
#pragma unroll
    for (int i = 0; i < 16; ++i) b.l[i] = 0;
    b.l[0] = (uint32_t)v;
    b.l[1] = (uint32_t)(v >> 32);
}
__device__ __forceinline__ void big_mul(Big &b, uint32_t m) {
    uint64_t carry = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const uint64_t x = (uint64_t)b.l[i] * m + carry;
        b.l[i] = (uint32_t)x;
        carry = x >> 32;
    }
}
__device__ __forceinline__ void big_mul_pow10(Big &b, int e) {
    while (e >= 9) {
        big_mul(b, 1000000000u);
        e -= 9;
    }
    uint32_t r = 1;
    for (int i = 0; i < e; ++i) r *= 10u;
    if (r != 1) big_mul(b, r);
}
__device__ __forceinline__ void big_shl(Big &b, int k) {
    const int words = k >> 5, bits = k & 31;
    for (int i = 15; i >= 0; --i) {
        const uint32_t hi = (i - words >= 0) ? b.l[i - words] : 0u;
        const uint32_t lo = (i - words - 1 >= 0) ? b.l[i - words - 1] : 0u;
        b.l[i] = bits ? ((hi << bits) | (lo >> (32 - bits))) : hi;
    }
}
__device__ __forceinline__ int big_cmp(const Big &a, const Big &b) {
    for (int i = 15; i >= 0; --i)
        if (a.l[i] != b.l[i]) return a.l[i] < b.l[i] ? -1 : 1;
    return 0;
}

// A positive float (bit pattern; 0x7f800000 stands for 2^128) as S * 2^e with S integral.
__device__ __forceinline__ void float_parts(uint32_t bits, uint64_t &S, int &e) {
    if (bits >= 0x7f800000u) {
        S = 1ull << 23;
        e = 105;
        return;
    }
    const uint32_t ex = bits >> 23, man = bits & 0x7fffffu;
    if (ex == 0) {
        S = man;
        e = -149;
    } else {
        S = man | 0x800000u;
        e = (int)ex - 150;
    }
}

// Sign of w * 10^q - (midpoint of the adjacent floats lo_bits, lo_bits + 1).  Rarely taken;
// kept out of line so the common path keeps few registers.
__device__ __noinline__ int cmp_midpoint(uint64_t w, int q, uint32_t lo_bits) {
    uint64_t S1, S2;
    int e1, e2;
    float_parts(lo_bits, S1, e1);
    float_parts(lo_bits + 1, S2, e2);
    const int emin = min(e1, e2);
    const uint64_t M = (S1 << (e1 - emin)) + (S2 << (e2 - emin));
    const int E = emin - 1;
    Big A, B;
    big_set(A, w);
    big_set(B, M);
    if (q >= 0)
        big_mul_pow10(A, q);
    else
        big_mul_pow10(B, -q);
    if (E >= 0)
        big_shl(B, E);
    else
        big_shl(A, -E);
    return big_cmp(A, B);
}

// Correctly rounded (to nearest, ties to even) float of w * 10^q, w >= 1.
__device__ float decimal_to_float(uint64_t w, int q) {
    if (q > 39) return __int_as_float(0x7f800000);  // >= 1e40
    if (q < -65) return 0.f;                         // < 1e-46, below half the least subnormal
    if (w <= (1ull << 24) && q >= -10 && q <= 10) {
        const float fw = (float)w;  // exact
        return q >= 0 ? __fmul_rn(fw, pow10f_exact(q)) : __fdiv_rn(fw, pow10f_exact(-q));
    }
    double d;
    const bool exact_double = w <= (1ull << 53) && q >= -22 && q <= 22;
    if (exact_double) {
        d = q >= 0 ? __dmul_rn((double)w, pow10d_exact(q)) : __ddiv_rn((double)w, pow10d_exact(-q));
    } else {
        d = (double)w;
        int e = q;
        while (e > 0) {
            const int s = min(e, 22);
            d *= pow10d_exact(s);
            e -= s;
        }
        while (e < 0) {
            const int s = min(-e, 22);
            d /= pow10d_exact(s);
            e += s;
        }
    }
    const float f0 = __double2float_rn(d);
    uint32_t b0 = __float_as_uint(f0);
    if (exact_double) {
        // d is w * 10^q rounded once; rounding d to float is exact unless d is a midpoint.
        const double two103 = (double)(1ull << 52) * (double)(1ull << 51);
        double mid;
        if (b0 >= 0x7f800000u) {
            mid = (double)__uint_as_float(0x7f7fffffu) + two103;  // FLT_MAX + half its ulp
        } else {
            const double df = (double)f0;
            if (df == d) return f0;
            const uint32_t nb = d > df ? b0 + 1 : b0 - 1;
            mid = nb >= 0x7f800000u ? df + two103 : 0.5 * (df + (double)__uint_as_float(nb));
        }
        if (d != mid) return f0;
    }
    if (b0 >= 0x7f800000u) b0 = 0x7f7fffffu;
    int c = cmp_midpoint(w, q, b0);
    if (c > 0) return __uint_as_float(b0 + 1);  // 0x7f800000 = inf
    if (c == 0) return __uint_as_float((b0 & 1u) ? b0 + 1 : b0);
    if (b0 == 0) return 0.f;
    c = cmp_midpoint(w, q, b0 - 1);
    if (c < 0) return __uint_as_float(b0 - 1);
    if (c == 0) return __uint_as_float((b0 & 1u) ? b0 - 1 : b0);
    return __uint_as_float(b0);
}

// ---- token parsers ---------------------------------------------------------------------

__device__ __forceinline__ uint32_t at(const unsigned char *t, int64_t i, int64_t len) {
    return i < len ? (uint32_t)__ldg(t + i) : 32u;  // past the end reads as a space
}

// %d: [+-]digits, within int32.  Returns 0 or a failure reason.
__device__ __forceinline__ uint32_t parse_int(const unsigned char *t, int64_t i, int64_t len, int32_t *out) {
    uint32_t c = at(t, i, len);
    bool neg = false;
    if (c == '+' || c == '-') {
        neg = c == '-';
        c = at(t, ++i, len);
    }
    int64_t v = 0;
    int nd = 0;
    for (; !is_space(c); c = at(t, ++i, len)) {
        if (c < '0' || c > '9') return kBadInt;
        v = v * 10 + (int64_t)(c - '0');
        if (v > 2147483648ll) return kBadIntRange;
        if (++nd > kMaxToken) return kBadLong;
    }
    if (nd == 0) return kBadInt;
    if (neg) v = -v;
    if (v > 2147483647ll) return kBadIntRange;
    *out = (int32_t)v;
    return 0;
}

__device__ __forceinline__ uint32_t lower(uint32_t c) { return (c >= 'A' && c <= 'Z') ? c + 32u : c; }

// %f: [+-](digits[.digits]|.digits)([eE][+-]digits) | [+-](inf|infinity|nan).
__device__ __forceinline__ uint32_t parse_float(const unsigned char *t, int64_t i, int64_t len, float *out) {
    uint32_t c = at(t, i, len);
    bool neg = false;
    if (c == '+' || c == '-') {
        neg = c == '-';
        c = at(t, ++i, len);
    }
    const uint32_t lc = lower(c);
    if (lc == 'i' || lc == 'n') {
        char word[9];
        int n = 0;
        for (; !is_space(c) && n < 9; c = at(t, ++i, len)) word[n++] = (char)lower(c);
        if (!is_space(c)) return kBadFloat;
        auto eq = [&](const char *s) {
            int k = 0;
            for (; s[k]; ++k)
                if (k >= n || word[k] != s[k]) return false;
            return k == n;
        };
        if (eq("inf") || eq("infinity")) {
            *out = __int_as_float(neg ? (int)0xff800000u : 0x7f800000);
            return 0;
        }
        if (eq("nan")) {
            *out = __int_as_float(neg ? (int)0xffc00000u : 0x7fc00000);
            return 0;
        }
        return kBadFloat;
    }
    uint64_t w = 0;
    int nsig = 0, ndig = 0, nchars = 0;
    int64_t dexp = 0;
    bool point = false, trunc = false;
    for (; !is_space(c); c = at(t, ++i, len)) {
        if (++nchars > kMaxToken) return kBadLong;
        if (c == '.') {
            if (point) return kBadFloat;
            point = true;
            continue;
        }
        if (c < '0' || c > '9') break;
        ++ndig;
        const uint32_t d = c - '0';
        if (nsig < 19) {
            if (w != 0 || d != 0) {
                w = w * 10 + d;
                ++nsig;
            }
            if (point) --dexp;
        } else {
            if (d != 0) trunc = true;
            if (!point) ++dexp;
        }
    }
    if (ndig == 0) return kBadFloat;
    int64_t ex = 0;
    if (c == 'e' || c == 'E') {
        c = at(t, ++i, len);
        bool eneg = false;
        if (c == '+' || c == '-') {
            eneg = c == '-';
            c = at(t, ++i, len);
        }
        int ne = 0;
        for (; !is_space(c); c = at(t, ++i, len)) {
            if (c < '0' || c > '9') return kBadFloat;
            if (ex < 1000000) ex = ex * 10 + (c - '0');
            if (++ne > kMaxToken) return kBadLong;
        }
        if (ne == 0) return kBadFloat;
        if (eneg) ex = -ex;
    }
    if (!is_space(c)) return kBadFloat;
    float f = 0.f;
    if (w != 0) {
        int64_t q64 = dexp + ex;
        q64 = q64 > 100000 ? 100000 : (q64 < -100000 ? -100000 : q64);
        const int q = (int)q64;
        f = decimal_to_float(w, q);
        if (trunc && __float_as_uint(decimal_to_float(w + 1, q)) != __float_as_uint(f)) return kBadDigits;
    }
    *out = neg ? -f : f;
    return 0;
}

// The general parse of the token at byte i: (failure reason << 32) | the field's 32 bits.
// Out of line, so the short-token path of parse_tokens_kernel keeps few registers.
__device__ __noinline__ uint64_t parse_general(const unsigned char *t, int64_t i, int64_t len, bool is_rating) {
    uint32_t reason, word;
    if (is_rating) {
        float f = 0.f;
        reason = parse_float(t, i, len, &f);
        word = __float_as_uint(f);
    } else {
        int32_t v = 0;
        reason = parse_int(t, i, len, &v);
        word = (uint32_t)v;
    }
    return ((uint64_t)reason << 32) | word;
}

// carry: tokens before this text (chunks of a longer text; NULL = none); byte_base: the text's
// offset in the whole input, for error positions.
//
// The block's 16 KB of text and a 64-byte halo are staged in shared memory with coalesced
// 16-byte loads (bytes at or past len read as spaces).  Two passes over the blocks:
//   - kGeneral = false: every token is offered to the byte-parallel converter on the 8 bytes at
//     its start (text_token.h) and stored when taken; block_flags[b] records whether block b
//     holds a token it did not take.  No call, 32 registers, 8 blocks per SM.
//   - kGeneral = true: flagged blocks only; their remaining tokens are parsed by parse_int /
//     parse_float from global memory, and failures are reported through `bad`.
template <bool kGeneral>
__global__ void __launch_bounds__(kTB, kGeneral ? 4 : 8)
parse_tokens_kernel(const unsigned char *__restrict__ t, int64_t start, int64_t len,
                    const unsigned long long *block_base, uint32_t *out_words, unsigned long long cap_tokens,
                    unsigned long long *bad, const unsigned long long *carry, int64_t byte_base,
                    uint32_t *block_flags) {
    if (kGeneral && block_flags[blockIdx.x] == 0) return;
    __shared__ __align__(16) unsigned char s_text[kStage];
    const int64_t blk0 = (int64_t)blockIdx.x * kBlockBytes;
    for (int q = threadIdx.x; q < kStage / 16; q += kTB) {
        const int64_t g = blk0 + 16 * (int64_t)q;
        uint4 v;
        if (g + 16 <= len) {
            v = __ldg(reinterpret_cast<const uint4 *>(t + g));
        } else {
            uint32_t w[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                w[k] = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int64_t i = g + 4 * k + b;
                    w[k] |= (i < len ? (uint32_t)__ldg(t + i) : 32u) << (8 * b);
                }
            }
            v = make_uint4(w[0], w[1], w[2], w[3]);
        }
        *reinterpret_cast<uint4 *>(s_text + 16 * q) = v;
    }
    __syncthreads();

    const int base = threadIdx.x * kSeg;
    const int64_t seg = blk0 + base;
    uint64_t starts = 0, ns = 0;  // token starts; non-space bytes of [start, len)
    if (seg < len && seg + kSeg > start) {
        const uint4 *p = reinterpret_cast<const uint4 *>(s_text + base);
#pragma unroll
        for (int w = 0; w < 4; ++w) ns |= nonspace16(p[w]) << (16 * w);
        if (start > seg) ns &= (start - seg >= kSeg) ? 0ull : (~0ull << (start - seg));
        const uint32_t before = base > 0 ? (uint32_t)s_text[base - 1] : (seg > 0 ? (uint32_t)__ldg(t + seg - 1) : 32u);
        const uint64_t prev = (seg - 1 >= start && !is_space(before)) ? 1ull : 0ull;
        starts = ns & ~((ns << 1) | prev);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // Non-space bytes of the next segment (its first 16 bytes are enough for tokens of up to 7
    // characters): the next lane's mask, or for the last lane the staged bytes after its own
    // (base + 80 <= kStage).  Bytes there before `start` cannot follow a token of this segment.
    uint64_t ns_next = __shfl_down_sync(0xffffffffu, ns, 1);
    if (lane == 31) ns_next = nonspace16(*reinterpret_cast<const uint4 *>(s_text + base + kSeg));
    const unsigned c = (unsigned)__popcll(starts);
    // Block-wide exclusive scan of the per-thread counts.
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
    }
    __shared__ unsigned s_w[kTB / 32];
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    unsigned wbase = 0;
    for (int w = 0; w < warp; ++w) wbase += s_w[w];
    unsigned long long tok = block_base[blockIdx.x] + wbase + (incl - c) + (carry ? *carry : 0ull);
    int field = (int)(tok % 3ull);
    bool left = false;  // a token the byte-parallel converter did not take
    const uint32_t *s32 = reinterpret_cast<const uint32_t *>(s_text);
    while (starts) {
        const int j = __ffsll((long long)starts) - 1;
        starts &= starts - 1;
        // The 8 bytes at the token's start (p + 12 <= kStage: p < kBlockBytes).
        const int p = base + j;
        const uint32_t a = s32[p >> 2], b = s32[(p >> 2) + 1], c2 = s32[(p >> 2) + 2];
        const int sh = (p & 3) * 8;
        const uint64_t x = ((uint64_t)__funnelshift_r(b, c2, sh) << 32) | __funnelshift_r(a, b, sh);
        // Token length: the first space in the 8 bytes (none: 8 or more characters).
        const uint32_t after = (uint32_t)(j ? (ns >> j) | (ns_next << (64 - j)) : ns);
        const uint32_t spaces = ~after & 0xffu;
        uint32_t word = 0;
        const bool taken = spaces != 0 && text_token::convert_n(x, __ffs(spaces) - 1, field == 2, &word);
        if (!kGeneral) {
            if (taken && tok < cap_tokens) out_words[tok] = word;
            left |= !taken;
        } else if (!taken) {
            const int64_t i = seg + j;
            const uint64_t r = parse_general(t, i, len, field == 2);
            const uint32_t reason = (uint32_t)(r >> 32);
            if (reason == 0 && tok < cap_tokens) out_words[tok] = (uint32_t)r;
            if (reason != 0) atomicMin(bad, ((unsigned long long)(i + byte_base) << 8) | reason);
        }
        ++tok;
        field = field == 2 ? 0 : field + 1;
    }
    if (!kGeneral) {
        const int any = __syncthreads_or(left ? 1 : 0);
        if (threadIdx.x == 0) block_flags[blockIdx.x] = (uint32_t)any;
    }
}

// Both passes of the parse over nb blocks of 16 KB.
void launch_parse(const unsigned char *t, int64_t start, int64_t len, int64_t nb, const unsigned long long *block_base,
                  uint32_t *out_words, unsigned long long cap_tokens, unsigned long long *bad,
                  const unsigned long long *carry, int64_t byte_base, uint32_t *block_flags, cudaStream_t s) {
    parse_tokens_kernel<false><<<(unsigned)nb, kTB, 0, s>>>(t, start, len, block_base, out_words, cap_tokens, bad,
                                                            carry, byte_base, block_flags);
    parse_tokens_kernel<true><<<(unsigned)nb, kTB, 0, s>>>(t, start, len, block_base, out_words, cap_tokens, bad,
                                                           carry, byte_base, block_flags);
}

// After a chunk: carry += the chunk's token count (counts[nb]); host_carry receives it.
__global__ void advance_carry_kernel(unsigned long long *carry, const unsigned long long *chunk_total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *carry += *chunk_total;
}

const char *reason_text(uint32_t r) {
    switch (r) {
        case kBadInt: return "malformed integer id";
        case kBadIntRange: return "id outside the int32 range";
        case kBadFloat: return "malformed rating";
        case kBadDigits: return "rating needs more than 19 significant digits to round";
        case kBadLong: return "token longer than 1024 characters";
        default: return "malformed token";
    }
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

struct StreamBuf {
    cudaStream_t s;
    void *p = nullptr;
    explicit StreamBuf(cudaStream_t st) : s(st) {}
    ~StreamBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

}  // namespace

// Offset of the first byte after `lines` header lines, as fscanf(f, "%[^\n]\n", line) called
// `lines` times consumes them (transform.cpp:31-33): a call reads the rest of a non-empty line
// and then all whitespace; on an empty line or at the end it fails and so do the next ones.
int64_t text_data_start(const unsigned char *p, int64_t len, int lines) {
    int64_t i = 0;
    for (int h = 0; h < lines; ++h) {
        if (i >= len || p[i] == '\n') break;
        while (i < len && p[i] != '\n') ++i;
        while (i < len && (p[i] == ' ' || (p[i] >= '\t' && p[i] <= '\r'))) ++i;
    }
    return i;
}

// Parses the device text into records.  d_out == NULL (or cap too small) returns the count only.
int parse_text_device(const unsigned char *d_text, int64_t len, int64_t start, cumf_node *d_out, int64_t cap,
                      int64_t *n_records, cudaStream_t s) {
    if (!n_records || len < 0 || start < 0 || cap < 0 || (len > 0 && !d_text))
        return fail(CUMF_ERR_ARG, "parse_text: bad arguments");
    if (reinterpret_cast<uintptr_t>(d_text) & 15u) return fail(CUMF_ERR_ARG, "parse_text: text must be 16-byte aligned");
    *n_records = 0;
    if (start >= len) return CUMF_OK;
    const int64_t nb = (len + kBlockBytes - 1) / kBlockBytes;
    if (nb > 0x7fffffffll) return fail(CUMF_ERR_ARG, "parse_text: text too large");
    // Stream-ordered scratch: block counts, then the total, then the first-bad word, then the
    // block flags of the parse.
    StreamBuf scratch(s);
    CUMF_CUDA(cudaMallocAsync(&scratch.p, (size_t)(nb + 2) * sizeof(unsigned long long) + (size_t)nb * 4, s));
    unsigned long long *counts = static_cast<unsigned long long *>(scratch.p);
    unsigned long long *bad = counts + nb + 1;
    uint32_t *flags = reinterpret_cast<uint32_t *>(counts + nb + 2);
    count_tokens_kernel<<<(unsigned)nb, kTB, 0, s>>>(d_text, start, len, counts);
    scan_blocks_kernel<<<1, kScanThreads, 0, s>>>(counts, nb);
    CUMF_CUDA(cudaGetLastError());
    unsigned long long tail[2] = {0, ~0ull};  // total tokens, first bad token
    if (d_out) {
        // Parse in the same pass; records past `cap` are parsed (for errors) but not stored.
        CUMF_CUDA(cudaMemsetAsync(bad, 0xff, sizeof(unsigned long long), s));
        launch_parse(d_text, start, len, nb, counts, reinterpret_cast<uint32_t *>(d_out), (unsigned long long)cap * 3ull,
                     bad, nullptr, 0, flags, s);
        CUMF_CUDA(cudaGetLastError());
        CUMF_CUDA(cudaMemcpyAsync(tail, counts + nb, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    } else {
        CUMF_CUDA(cudaMemcpyAsync(tail, counts + nb, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    }
    CUMF_CUDA(cudaStreamSynchronize(s));
    const unsigned long long total = tail[0];
    if (total % 3 != 0)
        return fail(CUMF_ERR_FORMAT, "parse_text: " + std::to_string(total) +
                                         " tokens do not form whole (u, v, r) records");
    *n_records = (int64_t)(total / 3);
    if (tail[1] != ~0ull)
        return fail(CUMF_ERR_FORMAT, "parse_text: byte " + std::to_string(tail[1] >> 8) + ": " +
                                         reason_text((uint32_t)(tail[1] & 0xffu)));
    if (d_out && cap < *n_records)
        return fail(CUMF_ERR_ARG, "parse_text: output holds " + std::to_string(cap) + " records, " +
                                      std::to_string(*n_records) + " needed");
    return CUMF_OK;
}

// Host text -> host records with the copies overlapped: chunks of about 64 MB, each
// starting right after a whitespace byte (no token crosses a boundary), go H2D on one stream,
// are counted, scanned and parsed on another, and the records completed so far go D2H on a
// third while later chunks are still arriving.  Token indices continue across chunks through
// a device carry, so a record may span two chunks.
int parse_text_host(const unsigned char *h_text, int64_t len, int64_t start, cumf_node *h_out, int64_t cap,
                    int64_t *n_records) {
    constexpr int64_t kChunk = 64ll << 20;
    *n_records = 0;
    if (start >= len) return CUMF_OK;
    std::vector<int64_t> bounds{start};
    while (bounds.back() < len) {
        int64_t b = std::min(len, bounds.back() + kChunk);
        while (b < len && !(h_text[b - 1] == ' ' || (h_text[b - 1] >= '\t' && h_text[b - 1] <= '\r'))) ++b;
        bounds.push_back(b);
    }
    const int chunks = (int)bounds.size() - 1;
    int64_t max_chunk = 0;
    for (int c = 0; c < chunks; ++c) max_chunk = std::max(max_chunk, bounds[c + 1] - bounds[c]);
    const int64_t max_nb = (max_chunk + kBlockBytes - 1) / kBlockBytes;
    const int64_t rec_cap = (len - start) / 6 + 2;  // tokens are at least 2 bytes apart
    struct Dev {
        void *p = nullptr;
        ~Dev() {
            if (p) cudaFree(p);
        }
    } slot[2], counts[2], recs, small;
    struct Stm {
        cudaStream_t s = nullptr;
        ~Stm() {
            if (s) cudaStreamDestroy(s);
        }
    } h2d, comp, d2h;
    struct Evs {
        std::vector<cudaEvent_t> e;
        ~Evs() {
            for (cudaEvent_t x : e) cudaEventDestroy(x);
        }
        cudaEvent_t make() {
            cudaEvent_t x = nullptr;
            if (cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess) e.push_back(x);
            return x;
        }
    } evs;
    struct PinnedCarry {
        unsigned long long *p = nullptr;
        ~PinnedCarry() {
            if (p) cudaFreeHost(p);
        }
    } hc;
    for (int k = 0; k < 2; ++k) {
        CUMF_CUDA(cudaMalloc(&slot[k].p, (size_t)max_chunk + 16));
        // block counts and the total, then the parse's block flags
        CUMF_CUDA(cudaMalloc(&counts[k].p, (size_t)(max_nb + 1) * sizeof(unsigned long long) + (size_t)max_nb * 4));
    }
    CUMF_CUDA(cudaMalloc(&recs.p, (size_t)rec_cap * sizeof(cumf_node)));
    CUMF_CUDA(cudaMalloc(&small.p, 2 * sizeof(unsigned long long)));  // carry, first bad token
    CUMF_CUDA(cudaMallocHost(&hc.p, (size_t)(chunks + 1) * sizeof(unsigned long long)));
    unsigned long long *carry = static_cast<unsigned long long *>(small.p), *bad = carry + 1;
    CUMF_CUDA(cudaStreamCreateWithFlags(&h2d.s, cudaStreamNonBlocking));
    CUMF_CUDA(cudaStreamCreateWithFlags(&comp.s, cudaStreamNonBlocking));
    CUMF_CUDA(cudaStreamCreateWithFlags(&d2h.s, cudaStreamNonBlocking));
    CUMF_CUDA(cudaMemsetAsync(carry, 0, sizeof(unsigned long long), comp.s));
    CUMF_CUDA(cudaMemsetAsync(bad, 0xff, sizeof(unsigned long long), comp.s));
    std::vector<cudaEvent_t> copied(chunks), parsed(chunks);
    for (int c = 0; c < chunks; ++c) {
        copied[c] = evs.make();
        parsed[c] = evs.make();
        if (!copied[c] || !parsed[c]) return fail(CUMF_ERR_CUDA, "parse_text_host: events");
    }
    int64_t sent = 0;  // records already copied back
    uint32_t *words = static_cast<uint32_t *>(recs.p);
    const unsigned long long cap_tokens = (unsigned long long)rec_cap * 3ull;
    auto flush_done = [&](int c) -> int {  // copy back the records completed by chunk c
        CUMF_CUDA(cudaEventSynchronize(parsed[c]));
        const int64_t done = (int64_t)(hc.p[c + 1] / 3ull);
        const int64_t upto = std::min(done, cap);
        if (h_out && upto > sent) {
            CUMF_CUDA(cudaMemcpyAsync(h_out + sent, static_cast<cumf_node *>(recs.p) + sent,
                                      (size_t)(upto - sent) * sizeof(cumf_node), cudaMemcpyDeviceToHost, d2h.s));
            sent = upto;
        }
        return CUMF_OK;
    };
    for (int c = 0; c < chunks; ++c) {
        const int k = c & 1;
        const int64_t clen = bounds[c + 1] - bounds[c];
        const int64_t nb = (clen + kBlockBytes - 1) / kBlockBytes;
        if (c >= 2) CUMF_CUDA(cudaStreamWaitEvent(h2d.s, parsed[c - 2], 0));  // the slot is free again
        CUMF_CUDA(cudaMemcpyAsync(slot[k].p, h_text + bounds[c], (size_t)clen, cudaMemcpyHostToDevice, h2d.s));
        CUMF_CUDA(cudaEventRecord(copied[c], h2d.s));
        CUMF_CUDA(cudaStreamWaitEvent(comp.s, copied[c], 0));
        const unsigned char *t = static_cast<const unsigned char *>(slot[k].p);
        unsigned long long *cnt = static_cast<unsigned long long *>(counts[k].p);
        count_tokens_kernel<<<(unsigned)nb, kTB, 0, comp.s>>>(t, 0, clen, cnt);
        scan_blocks_kernel<<<1, kScanThreads, 0, comp.s>>>(cnt, nb);
        launch_parse(t, 0, clen, nb, cnt, words, cap_tokens, bad, carry, bounds[c],
                     reinterpret_cast<uint32_t *>(cnt + max_nb + 1), comp.s);
        advance_carry_kernel<<<1, 32, 0, comp.s>>>(carry, cnt + nb);
        CUMF_CUDA(cudaGetLastError());
        CUMF_CUDA(cudaMemcpyAsync(hc.p + c + 1, carry, sizeof(unsigned long long), cudaMemcpyDeviceToHost, comp.s));
        CUMF_CUDA(cudaEventRecord(parsed[c], comp.s));
        if (c >= 1)  // chunk c is queued: copy back what chunk c - 1 completed meanwhile
            if (int rc = flush_done(c - 1)) return rc;
    }
    if (int rc = flush_done(chunks - 1)) return rc;
    unsigned long long first_bad = 0;
    CUMF_CUDA(cudaMemcpyAsync(&first_bad, bad, sizeof(first_bad), cudaMemcpyDeviceToHost, comp.s));
    CUMF_CUDA(cudaStreamSynchronize(comp.s));
    CUMF_CUDA(cudaStreamSynchronize(d2h.s));
    const unsigned long long total = hc.p[chunks];
    if (total % 3 != 0)
        return fail(CUMF_ERR_FORMAT, "parse_text: " + std::to_string(total) +
                                         " tokens do not form whole (u, v, r) records");
    *n_records = (int64_t)(total / 3);
    if (first_bad != ~0ull)
        return fail(CUMF_ERR_FORMAT, "parse_text: byte " + std::to_string(first_bad >> 8) + ": " +
                                         reason_text((uint32_t)(first_bad & 0xffu)));
    if (h_out && cap < *n_records)
        return fail(CUMF_ERR_ARG, "parse_text: output holds " + std::to_string(cap) + " records, " +
                                      std::to_string(*n_records) + " needed");
    return CUMF_OK;
}

namespace {

__global__ void extent_kernel(const cumf_node *__restrict__ R, int64_t nnz, int *d_ext) {
    int mu = 0, mv = 0, neg = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const int u = R[i].u, v = R[i].v;
        neg |= (u < 0) | (v < 0);
        mu = max(mu, u + 1);
        mv = max(mv, v + 1);
    }
    atomicMax(&d_ext[0], mu);
    atomicMax(&d_ext[1], mv);
    if (neg) atomicOr(&d_ext[2], 1);
}

// Reads a whole file into pinned memory (16 spare zero bytes at the end).
int read_text_file(const char *path, unsigned char **buf, int64_t *len) {
    *buf = nullptr;
    *len = 0;
    FILE *f = path ? fopen(path, "rb") : nullptr;
    if (!f) return fail(CUMF_ERR_IO, std::string("file ") + (path ? path : "(null)") + " open failed");
    struct stat st;
    if (fstat(fileno(f), &st) != 0) {
        fclose(f);
        return fail(CUMF_ERR_IO, std::string("cannot stat ") + path);
    }
    const int64_t n = (int64_t)st.st_size;
    unsigned char *p = nullptr;
    if (cudaMallocHost(&p, (size_t)n + 16) != cudaSuccess) {
        fclose(f);
        cudaGetLastError();
        return fail(CUMF_ERR_NOMEM, "cannot allocate pinned memory for " + std::string(path));
    }
    const size_t got = n ? fread(p, 1, (size_t)n, f) : 0;
    fclose(f);
    if ((int64_t)got != n) {
        cudaFreeHost(p);
        return fail(CUMF_ERR_IO, std::string("short read from ") + path);
    }
    memset(p + n, 0, 16);
    *buf = p;
    *len = n;
    return CUMF_OK;
}

// Host text -> device records (allocated here).
int text_to_device_records(const unsigned char *h_text, int64_t len, int header_lines, cumf_node **d_rec,
                           int64_t *n, cudaStream_t s) {
    *d_rec = nullptr;
    *n = 0;
    const int64_t start = text_data_start(h_text, len, header_lines);
    DevBuf text;
    CUMF_CUDA(cudaMalloc(&text.p, (size_t)len + 16));
    CUMF_CUDA(cudaMemcpyAsync(text.p, h_text, (size_t)len, cudaMemcpyHostToDevice, s));
    const unsigned char *dt = static_cast<const unsigned char *>(text.p);
    if (int rc = parse_text_device(dt, len, start, nullptr, 0, n, s)) return rc;
    if (*n == 0) return CUMF_OK;
    void *out = nullptr;
    CUMF_CUDA(cudaMalloc(&out, (size_t)*n * sizeof(cumf_node)));
    int64_t got = 0;
    if (int rc = parse_text_device(dt, len, start, static_cast<cumf_node *>(out), *n, &got, s)) {
        cudaFree(out);
        return rc;
    }
    *d_rec = static_cast<cumf_node *>(out);
    return CUMF_OK;
}

}  // namespace

}  // namespace cumf

using namespace cumf;

extern "C" int cumf_text_data_start(const char *text, int64_t len, int header_lines, int64_t *start) {
    if (!start || len < 0 || (len > 0 && !text) || header_lines < 0) return fail(CUMF_ERR_ARG, "bad text_data_start arguments");
    *start = text_data_start(reinterpret_cast<const unsigned char *>(text), len, header_lines);
    return CUMF_OK;
}

extern "C" int cumf_dev_parse_text(const void *d_text, int64_t len, int64_t start, cumf_node *d_out, int64_t cap,
                                   int64_t *n_records, void *stream) {
    return parse_text_device(static_cast<const unsigned char *>(d_text), len, start, d_out, cap, n_records,
                             static_cast<cudaStream_t>(stream));
}

extern "C" int cumf_read_text_problem(const char *path, int header_lines, int pinned, cumf_problem *out) {
    TraceRange trace("text parse: read text problem");
    if (!out || header_lines < 0) return fail(CUMF_ERR_ARG, "bad read_text_problem arguments");
    memset(out, 0, sizeof(*out));
    out->m = out->n = 1;
    unsigned char *h = nullptr;
    int64_t len = 0;
    if (int rc = read_text_file(path, &h, &len)) return rc;
    cudaStream_t s = nullptr;
    cumf_node *d = nullptr;
    int64_t n = 0;
    int rc = text_to_device_records(h, len, header_lines, &d, &n, s);
    cudaFreeHost(h);
    if (rc) return rc;
    DevBuf rec;
    rec.p = d;
    if ((rc = cumf_alloc_problem(n, pinned, out))) return rc;
    if (n > 0) {
        DevBuf ext;
        cudaError_t e = cudaMalloc(&ext.p, 3 * sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(ext.p, 0, 3 * sizeof(int), s);
        if (e == cudaSuccess) {
            const int blocks = (int)std::min<int64_t>(4096, (n + 255) / 256);
            extent_kernel<<<blocks, 256, 0, s>>>(d, n, static_cast<int *>(ext.p));
            e = cudaGetLastError();
        }
        int hext[3] = {0, 0, 0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(hext, ext.p, sizeof(hext), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->R, d, (size_t)n * sizeof(cumf_node), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cumf_free_problem(out);
            return cuda_fail(e, "read_text_problem");
        }
        if (hext[2]) {
            cumf_free_problem(out);
            return fail(CUMF_ERR_FORMAT, std::string("negative user or item id in ") + path);
        }
        out->m = std::max(1, hext[0]);
        out->n = std::max(1, hext[1]);
    }
    return CUMF_OK;
}

extern "C" int cumf_convert_text(const char *in_path, const char *out_path, int header_lines, int64_t *n_records) {
    if (header_lines < 0) return fail(CUMF_ERR_ARG, "bad convert_text arguments");
    if (n_records) *n_records = 0;
    unsigned char *h = nullptr;
    int64_t len = 0;
    if (int rc = read_text_file(in_path, &h, &len)) return rc;
    cudaStream_t s = nullptr;
    cumf_node *d = nullptr;
    int64_t n = 0;
    int rc = text_to_device_records(h, len, header_lines, &d, &n, s);
    cudaFreeHost(h);
    if (rc) return rc;
    DevBuf rec;
    rec.p = d;
    cumf_problem p;
    if ((rc = cumf_alloc_problem(n, 1, &p))) return rc;
    if (n > 0) {
        cudaError_t e = cudaMemcpyAsync(p.R, d, (size_t)n * sizeof(cumf_node), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cumf_free_problem(&p);
            return cuda_fail(e, "convert_text");
        }
    }
    const std::string dst = out_path ? std::string(out_path) : std::string(in_path) + ".bin";
    rc = cumf_write_problem(dst.c_str(), &p);
    cumf_free_problem(&p);
    if (rc == CUMF_OK && n_records) *n_records = n;
    return rc;
}

extern "C" int cumf_parse_text_host(const char *text, int64_t len, int header_lines, cumf_node *out, int64_t cap,
                                    int64_t *n_records) {
    TraceRange trace("text parse: host text, overlapped chunks");
    if (!n_records || len < 0 || (len > 0 && !text) || header_lines < 0 || cap < 0 || (out == nullptr && cap > 0))
        return fail(CUMF_ERR_ARG, "parse_text_host: bad arguments");
    const unsigned char *p = reinterpret_cast<const unsigned char *>(text);
    return parse_text_host(p, len, text_data_start(p, len, header_lines), out, cap, n_records);
}
