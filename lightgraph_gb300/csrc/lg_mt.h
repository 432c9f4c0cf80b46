// MT19937 and the float draws of the reference's RandGen (src/RandGen.h:16-44):
// one std::mt19937 per LightGraph iteration, seeded with 854123 + iteration,
// read through std::uniform_real_distribution<float>(0, 1).
//
// MT19937 is restated from its published definition (Matsumoto and
// Nishimura, 1998): 624-word state, recurrence offset 397, twist matrix
// 0x9908B0DF, tempering (11, 7/0x9D2C5680, 15/0xEFC60000, 18), initialised
// by x[i] = 1812433253 * (x[i-1] ^ (x[i-1] >> 30)) + i. The float draw is the
// C++ generate_canonical<float, 24> over one 32-bit output as libstdc++ (GCC 13)
// evaluates it: float(x) / 2^32, and the largest float below 1 when that
// rounds to 1; uniform_real_distribution(0, 1) then returns it unchanged.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define LG_MT_HD __host__ __device__ __forceinline__
#else
#define LG_MT_HD inline
#endif

namespace lg {

constexpr int kMtN = 624;
constexpr int kMtM = 397;

LG_MT_HD uint32_t mt_init_word(uint32_t prev, uint32_t i) { return 1812433253u * (prev ^ (prev >> 30)) + i; }

// New word i of a twist from the current words i and i+1 and the word
// 397 ahead (already renewed for i >= 227 in the sequential definition).
LG_MT_HD uint32_t mt_twist_word(uint32_t cur, uint32_t next, uint32_t ahead) {
    const uint32_t y = (cur & 0x80000000u) | (next & 0x7FFFFFFFu);
    return ahead ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
}

LG_MT_HD uint32_t mt_temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return y;
}

LG_MT_HD float mt_canonical_float(uint32_t x) {
    const float r = (float)x * 2.3283064365386963e-10f;  // exact scaling by 2^-32
    return r >= 1.0f ? 0.99999994039535522f : r;         // largest float below 1
}

// Sequential generator (host tests and reference-side checks).
struct Mt19937 {
    uint32_t x[kMtN];
    int i;
    explicit Mt19937(uint32_t seed) {
        x[0] = seed;
        for (int k = 1; k < kMtN; ++k) x[k] = mt_init_word(x[k - 1], (uint32_t)k);
        i = kMtN;
    }
    void twist() {
        for (int k = 0; k < kMtN; ++k) x[k] = mt_twist_word(x[k], x[(k + 1) % kMtN], x[(k + kMtM) % kMtN]);
        i = 0;
    }
    uint32_t next() {
        if (i >= kMtN) twist();
        return mt_temper(x[i++]);
    }
};

}  // namespace lg
