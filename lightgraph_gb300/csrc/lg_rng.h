// Counter-based random streams shared by every kernel of the LightGraph path.
//
// The reference draws its jitter from std::mt19937 engines whose state depends
// on how TBB splits the work (RandGen rng(1) per render chunk,
// src/Renderer.h:518; a shared engine in EnvLight, src/Light.h:189), so its
// images are not reproducible. Here every draw is a pure function of
// (seed, stream, draw key): the same pixel, sample and loop iteration always
// get the same number, whatever the launch shape or the other requests in
// flight. The CPU oracle restates these formulas to consume identical numbers.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define LG_HD __host__ __device__ __forceinline__
#else
#define LG_HD inline
#endif

namespace lg {

// Stream domains (top byte of the 64-bit stream id).
enum : uint64_t {
    kDomainPixel = 0x01ull << 56,   // id = pixel * spp + aa_sample
    kDomainVertex = 0x02ull << 56,  // id = graph << 32 | vertex
};

// Draw tags inside a stream (top nibble of the 32-bit draw key).
enum : uint32_t {
    kTagJitterX = 0x00000000u,
    kTagJitterY = 0x00000001u,
    kTagPrimarySpan = 0x10000000u,  // | span ordinal along the primary ray
    kTagPrimaryStep = 0x20000000u,  // | primary loop iteration
    kTagShadowRay = 0x30000000u,    // | primary loop iteration (sub-stream)
    kTagShadowSpan = 0x40000000u,   // | span ordinal along the shadow ray
    kTagShadowStep = 0x50000000u,   // | shadow loop iteration
    kTagEnvU = 0x60000000u,
    kTagEnvV = 0x60000001u,
};

LG_HD uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

LG_HD uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

// Uniform float in [0, 1) with 24 random bits.
LG_HD float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }

// Key of one stream.
struct Stream {
    uint32_t a, b;
};

LG_HD Stream make_stream(uint64_t seed, uint64_t stream_id) {
    const uint64_t k = mix64(seed ^ mix64(stream_id));
    Stream s;
    s.a = (uint32_t)k;
    s.b = (uint32_t)(k >> 32);
    return s;
}

// Draw number `key` of stream s.
// The key is spread by an odd multiplier (a bijection) before the one hash,
// so consecutive keys of a stream give independent-looking draws.
LG_HD float draw(Stream s, uint32_t key) { return u01(hash32(s.a ^ (s.b + key * 0x9E3779B9u))); }

// Sub-stream of a shadow ray: keyed by the primary iteration n, light k and
// light sample ls (render), or by light k and sample ls with n = 0 (vertices).
// The key splits into a per-iteration part (s.a and shadow_iter_word(s, n))
// and the light terms, so a caller can carry the two words instead of the
// stream and the iteration.
LG_HD uint32_t shadow_iter_word(Stream s, uint32_t n) { return hash32(s.b ^ (kTagShadowRay | (n & 0x0FFFFFFFu))); }
LG_HD uint32_t shadow_key_from(uint32_t sa, uint32_t iter_word, uint32_t k, uint32_t ls) {
    return hash32(sa ^ (iter_word + k * 0x9E3779B9u + ls * 0x85EBCA6Bu));
}
LG_HD uint32_t shadow_key(Stream s, uint32_t n, uint32_t k, uint32_t ls) {
    return shadow_key_from(s.a, shadow_iter_word(s, n), k, ls);
}

LG_HD float draw_sub(uint32_t sub, uint32_t key) { return u01(hash32(sub ^ (key * 0x9E3779B9u))); }

// Step-jitter stream of one march. The jitter drawn at loop iteration q is
// the state after q + 1 steps of a full-period 32-bit linear congruential
// generator seeded with a hash of the march's key. Every iteration advances
// it, whether its sample is taken or not, so the number drawn at an
// iteration does not depend on earlier skip decisions (which FP32 and FP64
// can resolve differently). Its top 23 bits give u = (x >> 9) / 2^23.
constexpr uint32_t kStepLcgA = 1664525u, kStepLcgC = 1013904223u;
LG_HD uint32_t step_seed_primary(Stream s) { return hash32(s.a ^ (s.b + kTagPrimaryStep * 0x9E3779B9u)); }
LG_HD uint32_t step_seed_shadow(uint32_t sub) { return hash32(sub ^ kTagShadowStep); }
LG_HD uint32_t step_next(uint32_t x) { return x * kStepLcgA + kStepLcgC; }

}  // namespace lg
