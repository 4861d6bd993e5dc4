// glibc_shuffle.h - bit-exact, state-local replay of `srand(seed); random_shuffle(v)`.
//
// The reference builds its id permutations with srand(time(NULL)) followed by libstdc++
// std::random_shuffle over the identity (singleGPU/sgd.cu:39-53), and orders the u x v and
// x x y blocks of modes B/C with further random_shuffle calls (singleGPU/sgd_kernel.cu:263,
// 267, 411-431).  Layout parity for a given seed therefore needs the exact glibc rand()
// stream.  This file restates the published algorithms so the library never touches the
// process-wide rand() state:
//  - glibc random()/rand() with the default TYPE_3 state (degree 31, separation 3): the
//    additive lagged-Fibonacci generator r[i] = r[i-3] + r[i-31] (mod 2^32) seeded by the
//    Park-Miller minimal standard LCG (16807, mod 2^31-1, Schrage's factorisation), the
//    first 310 outputs discarded, each output r >> 1.  Described in P. Selinger, "The GLIBC
//    pseudo-random number generator" (2007).
//  - libstdc++ random_shuffle(first, last): for i = 1..n-1, j = rand() % (i+1), swap(a[i], a[j]).
#pragma once
#include <stdint.h>
#include <stddef.h>

namespace cumf {

class GlibcRand {
  public:
    explicit GlibcRand(uint32_t seed) { reseed(seed); }

    void reseed(uint32_t seed) {
        int32_t r[34];
        int32_t s = (int32_t)(seed == 0 ? 1u : seed);
        r[0] = s;
        for (int i = 1; i < 31; ++i) {
            // 16807 * r[i-1] mod (2^31 - 1), Schrage: 2^31-1 = 16807*127773 + 2836
            int64_t hi = r[i - 1] / 127773;
            int64_t lo = r[i - 1] % 127773;
            int64_t word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            r[i] = (int32_t)word;
        }
        for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
        for (int i = 0; i < 34; ++i) ring_[i] = (uint32_t)r[i];
        pos_ = 34;
        for (int i = 34; i < 344; ++i) step();
    }

    // Next value of rand(): in [0, 2^31).
    int32_t next() { return (int32_t)(step() >> 1); }

  private:
    // ring_ holds the last 34 words; word i = word(i-31) + word(i-3).
    uint32_t step() {
        uint32_t w = ring_[(pos_ - 31) % 34] + ring_[(pos_ - 3) % 34];
        ring_[pos_ % 34] = w;
        ++pos_;
        return w;
    }
    uint32_t ring_[34];
    uint64_t pos_;
};

template <typename T>
inline void glibc_random_shuffle(T *a, int64_t n, GlibcRand &rng) {
    for (int64_t i = 1; i < n; ++i) {
        int64_t j = (int64_t)rng.next() % (i + 1);
        if (j != i) {
            T t = a[i];
            a[i] = a[j];
            a[j] = t;
        }
    }
}

}  // namespace cumf
