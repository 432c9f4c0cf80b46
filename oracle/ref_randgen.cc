// Test infrastructure: exposes the reference's own RandGen (src/RandGen.h of
// asiroisvigneux/LightGraph, compiled from the reference tree where it lies;
// see oracle/build_ref.py) through a C entry point, so the tests can pin the
// oracle's random sequence to the reference's code. RandGen.h includes
// nothing itself; it needs <random> and <vector> before it.
#include <cstddef>
#include <cstdint>
#include <random>
#include <vector>

#include "RandGen.h"

// n draws of RandGen(iter)(id): the uniform [0, 1) floats scatterPoints
// consumes for iteration `id` (src/LightGraph.h:206-274).
extern "C" int lgr_randgen_draws(uint64_t iter, uint64_t id, int64_t n, float* out) {
    if (id >= iter || n < 0 || (n > 0 && !out)) return 1;
    RandGen rng((size_t)iter);
    for (int64_t k = 0; k < n; ++k) out[k] = rng((size_t)id);
    return 0;
}
