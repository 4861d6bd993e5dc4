// text_token.h - byte-parallel conversion of short rating-text tokens.
//
// Most tokens of a rating text are short: ids of up to 7 digits and ratings such as "4" or
// "3.5".  Such a token is converted from one 64-bit little-endian window of the text (byte 0 =
// the token's first character) with arithmetic on all 8 bytes at once.  The result equals what
// the general parsers of text_parse.cu give for the same token (%d, and %f correctly rounded);
// every token this path does not take (a sign, an exponent, inf/nan, 8 or more characters,
// any byte other than a digit or one '.', a '.' in an id) is left to them, and so are all
// errors.
//
// Shared by the device parser and host tests, so it uses no CUDA-only calls except the
// correctly rounded division, which is IEEE division on the host too.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define CUMF_HD __host__ __device__ __forceinline__
#else
#define CUMF_HD inline
#endif

namespace cumf {
namespace text_token {

constexpr uint64_t kOnes = 0x0101010101010101ull;
constexpr uint64_t kHigh = 0x8080808080808080ull;

CUMF_HD int lowest_byte(uint64_t high_bits) {  // index of the lowest byte whose bit 7 is set
#ifdef __CUDA_ARCH__
    return (__ffsll((long long)high_bits) - 8) >> 3;
#else
    return __builtin_ctzll(high_bits) >> 3;
#endif
}

CUMF_HD int popcount64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}

CUMF_HD bool space_byte(uint32_t c) { return c == 32u || (c - 9u) <= 4u; }

// Bit 7 of byte i is set iff byte i of x is zero.
CUMF_HD uint64_t zero_bytes(uint64_t x) { return ~(((x & ~kHigh) + ~kHigh) | x | ~kHigh); }

CUMF_HD float div_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

// Bit 7 of byte i is set iff byte i of x is a space (' ', '\t', '\n', '\v', '\f', '\r').
CUMF_HD uint64_t space_bytes(uint64_t x) {
    const uint64_t ascii = ~x & kHigh;
    const uint64_t ge9 = (x | kHigh) - 0x09ull * kOnes;      // bit 7: b >= 9
    const uint64_t gt13 = (x & ~kHigh) + 0x72ull * kOnes;    // bit 7: b >= 14
    return (zero_bytes(x ^ (0x20ull * kOnes)) | (ge9 & ~gt13 & ascii)) & kHigh;
}

// The bit 7 flags of the 8 bytes (as space_bytes gives them) -> an 8-bit mask, bit i = byte i.
CUMF_HD uint32_t byte_flags(uint64_t high_bits) { return (uint32_t)(((high_bits >> 7) * 0x0102040810204080ull) >> 56); }

// 4 digit values (0-9) in the bytes of a word, the most significant in byte 0 -> their number.
CUMF_HD uint32_t digits4(uint32_t d) {
    d = (d * 10u + (d >> 8)) & 0x00ff00ffu;  // byte 2j <- 10*b[2j] + b[2j+1]
    return (d * 100u + (d >> 16)) & 0xffffu;
}

// x: the 8 bytes starting at a token's first character; n (1..7): its length, byte n of x
// being a space.  is_rating: the token is the third field of a record (%f) rather than an id
// (%d).  Returns true and the 32-bit field (the id, or the float's bits) when the token is
// taken here.
CUMF_HD bool convert_n(uint64_t x, int n, bool is_rating, uint32_t *word) {
    uint64_t tmh = ((1ull << (8 * n)) - 1) & kHigh;  // bit 7 of each token byte
    const uint64_t dots = zero_bytes(x ^ (0x2eull * kOnes)) & tmh;
    // '0' <= b <= '9' per byte: b|0x80 - 0x30 keeps bit 7 iff b >= 0x30; (b&0x7f) + 0x46 sets it
    // iff b >= 0x3a; bytes >= 0x80 are excluded.
    const uint64_t digits = ((x | kHigh) - 0x30ull * kOnes) & ~((x & ~kHigh) + 0x46ull * kOnes) & ~x & kHigh;
    if (tmh & ~(digits | dots)) return false;
    uint64_t d = x;
    int nd = n, frac = 0;
    if (dots) {
        if (!is_rating || (dots & (dots - 1))) return false;  // '.' in an id, or two of them
        const uint64_t below = (dots >> 7) - 1;               // the bytes before the '.'
        d = (x & below) | ((x >> 8) & ~below);                // drop it
        nd = n - 1;
        frac = nd - lowest_byte(dots);
        if (nd == 0) return false;  // "." alone
    }
    // Digit values, the last one in byte 7 (leading zero bytes), then two 4-digit halves.
    const uint64_t dm = (1ull << (8 * nd)) - 1;
    const uint64_t v = ((d & dm) - (0x30ull * kOnes & dm)) << (64 - 8 * nd);
    const uint32_t value = digits4((uint32_t)v) * 10000u + digits4((uint32_t)(v >> 32));
    if (!is_rating) {
        *word = value;  // < 10^7
        return true;
    }
    // value < 10^7 < 2^24 and 10^frac (frac <= 6) are exact floats: one rounded division is
    // the correctly rounded value of value * 10^-frac (the general parser's first case does
    // the same).
    float f = (float)value;
    if (frac) f = div_rn(f, ((frac & 1) ? 10.f : 1.f) * ((frac & 2) ? 100.f : 1.f) * ((frac & 4) ? 10000.f : 1.f));
#ifdef __CUDA_ARCH__
    *word = __float_as_uint(f);
#else
    memcpy(word, &f, 4);
#endif
    return true;
}

// The same, finding the token's end in x itself (the first byte below 0x21 must be a space;
// a token of 8 or more characters is not taken).
CUMF_HD bool convert(uint64_t x, bool is_rating, uint32_t *word) {
    const uint64_t ctl = ~((x | kHigh) - 0x21ull * kOnes) & ~x & kHigh;
    const uint64_t end = ctl & (0ull - ctl);
    if (end == 0 || end == 0x80u || !(end & space_bytes(x))) return false;
    return convert_n(x, lowest_byte(end), is_rating, word);
}

}  // namespace text_token
}  // namespace cumf
