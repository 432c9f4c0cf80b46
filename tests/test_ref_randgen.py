"""The oracle's random sequence pinned to the reference's own code: the
reference's RandGen (src/RandGen.h), compiled from the reference tree by
oracle/build_ref.py, gives the same floats as the oracle's restatement
(std::mt19937 seeded 854123 + iteration through
std::uniform_real_distribution<float>), which the GPU dart thrower matches
bit for bit (tests/test_gpu_dart.py). Skips where the reference tree is
absent."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as po

REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                   "libref_randgen.so")


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF):
        pytest.skip("the reference tree is not present (oracle/_ref not built)")
    lib = C.CDLL(REF)
    lib.lgr_randgen_draws.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, C.c_void_p]
    lib.lgr_randgen_draws.restype = C.c_int
    return lib


@pytest.mark.parametrize("iter_, ids", [(1, [0]), (500, [0, 1, 37, 499])])
def test_oracle_draws_equal_reference_randgen(ref, iter_, ids):
    n = 20000
    for i in ids:
        out = np.zeros(n, np.float32)
        assert ref.lgr_randgen_draws(iter_, i, n, out.ctypes.data) == 0
        mine, _ = po.randgen_draws(854123 + i, n)
        assert np.array_equal(out.view(np.uint32), mine.view(np.uint32)), i
