// Host check of the byte-parallel token conversion (cumf_sgd_gb300/csrc/text_token.h) against
// strtol / strtof: every token it takes must be one the general parser accepts (%d: digits
// only; %f: digits with at most one '.') and convert to the same bits; every short well-formed
// token must be taken.  Built and run by tests/test_text_token.py.
#include "../../cumf_sgd_gb300/csrc/text_token.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

using namespace cumf::text_token;

static long checked = 0, taken = 0, bad = 0;

static bool all_digits(const std::string &t) {
    if (t.empty()) return false;
    for (char c : t)
        if (c < '0' || c > '9') return false;
    return true;
}

static bool decimal(const std::string &t) {  // digits with at most one '.', at least one digit
    int dots = 0, digits = 0;
    for (char c : t) {
        if (c == '.') ++dots;
        else if (c >= '0' && c <= '9') ++digits;
        else return false;
    }
    return dots <= 1 && digits >= 1;
}

static void check(const std::string &tok, char term, uint64_t filler) {
    unsigned char w[8];
    memcpy(w, &filler, 8);
    for (size_t i = 0; i < 8; ++i) {
        if (i < tok.size()) w[i] = (unsigned char)tok[i];
        else if (i == tok.size()) w[i] = (unsigned char)term;
    }
    uint64_t x;
    memcpy(&x, w, 8);
    const bool fits = tok.size() < 8;
    for (int rating = 0; rating < 2; ++rating) {
        uint32_t word = 0;
        const bool ok = convert(x, rating != 0, &word);
        // convert_n with the true length must agree with convert
        uint32_t word_n = 0;
        const bool ok_n = fits && !tok.empty() && convert_n(x, (int)tok.size(), rating != 0, &word_n);
        ++checked;
        const bool easy = fits && (rating ? decimal(tok) : all_digits(tok));
        if (ok != ok_n || (ok && word != word_n)) {
            if (bad < 10) fprintf(stderr, "convert/convert_n differ on '%s'\n", tok.c_str());
            ++bad;
        }
        if (!ok) {
            if (easy) {
                if (bad < 10) fprintf(stderr, "short well-formed token refused: '%s' (rating %d)\n", tok.c_str(), rating);
                ++bad;
            }
            continue;
        }
        ++taken;
        if (!easy) {
            if (bad < 10) fprintf(stderr, "token taken that the general parser rejects: '%s'\n", tok.c_str());
            ++bad;
            continue;
        }
        if (rating) {
            const float f = strtof(tok.c_str(), nullptr);
            uint32_t b;
            memcpy(&b, &f, 4);
            if (b != word) {
                if (bad < 10) fprintf(stderr, "'%s': %08x, strtof %08x\n", tok.c_str(), word, b);
                ++bad;
            }
        } else if ((uint32_t)strtol(tok.c_str(), nullptr, 10) != word) {
            if (bad < 10) fprintf(stderr, "'%s': %u, strtol %ld\n", tok.c_str(), word, strtol(tok.c_str(), nullptr, 10));
            ++bad;
        }
    }
}

int main() {
    std::mt19937_64 rng(5);
    static const char AL[] = {'0', '1', '5', '9', '.', '+', '-', 'e', '/', ':', '\x01', '\x80', '\xff', 'a', '7', '3'};
    static const char TERM[] = {' ', '\t', '\n', '\r', '\x0b', '\x0c'};
    const int A = (int)sizeof(AL);
    // every token of 1..5 characters over the alphabet
    for (int len = 1; len <= 5; ++len) {
        long total = 1;
        for (int i = 0; i < len; ++i) total *= A;
        for (long c = 0; c < total; ++c) {
            std::string s;
            long cc = c;
            for (int i = 0; i < len; ++i) {
                s.push_back(AL[cc % A]);
                cc /= A;
            }
            check(s, TERM[c % 6], rng());
        }
    }
    // random digit-heavy tokens of 1..9 characters, some with a stray symbol
    const char D[] = "0123456789.";
    for (long it = 0; it < 1000000; ++it) {
        const int len = 1 + (int)(rng() % 9);
        std::string s;
        for (int i = 0; i < len; ++i) s.push_back(rng() % 10 == 0 ? D[rng() % 11] : D[rng() % 10]);
        if (rng() % 50 == 0) s[rng() % len] = AL[rng() % A];
        check(s, TERM[rng() % 6], rng());
    }
    // values below 10^6 with a '.' at every position
    for (int v = 0; v < 1000000; v += (v < 20000 ? 1 : 7)) {
        const std::string s = std::to_string(v);
        for (size_t dp = 0; dp <= s.size(); ++dp) {
            const std::string t = s.substr(0, dp) + "." + s.substr(dp);
            if (t.size() <= 7) check(t, ' ', rng());
        }
        check(s, '\n', rng());
    }
    // the space mask of every byte value, and random words
    for (unsigned c = 0; c < 256; ++c) {
        const uint32_t f = byte_flags(space_bytes(c * kOnes));
        if (f != (space_byte(c) ? 0xffu : 0u)) {
            fprintf(stderr, "space mask of byte %u: %02x\n", c, f);
            ++bad;
        }
    }
    for (long it = 0; it < 2000000; ++it) {
        const uint64_t x = rng();
        uint32_t e = 0;
        for (int i = 0; i < 8; ++i)
            if (space_byte((uint32_t)(x >> (8 * i)) & 0xffu)) e |= 1u << i;
        if (byte_flags(space_bytes(x)) != e) ++bad;
    }
    printf("checked %ld taken %ld bad %ld\n", checked, taken, bad);
    return bad != 0;
}
