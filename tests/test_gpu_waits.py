"""Bounded device-side waits. The persistent Floyd-Warshall solves wait for
other items' results with a bounded number of polls and raise an error word
when a wait gives up, so a stalled queue ends its launch instead of hanging
the GPU. Here the same wait runs on a flag that nothing sets: it must give
up after its poll limit, report LG_ERR_TIMEOUT, and leave the context usable
(a persistent path solve afterwards matches the oracle, and its error word
reads clear)."""
import numpy as np
import pytest

from lightgraph_gb300 import _capi, scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up(gpu_ctx):
    lib = gpu_ctx.lib
    for polls in (1, 4096):
        assert lib.lg_wait_timeout_check(gpu_ctx.h, polls) == _capi.LG_ERR_TIMEOUT
    assert b"gave up" in lib.lg_last_error(gpu_ctx.h)
    # out-of-range limits are refused on the host, before any launch
    assert lib.lg_wait_timeout_check(gpu_ctx.h, 0) == _capi.LG_ERR_INVALID
    assert lib.lg_wait_timeout_check(gpu_ctx.h, (1 << 24) + 1) == _capi.LG_ERR_INVALID


def test_context_usable_after_a_wait_gave_up(gpu_ctx):
    lib = gpu_ctx.lib
    assert lib.lg_wait_timeout_check(gpu_ctx.h, 4096) == _capi.LG_ERR_TIMEOUT
    sc = scenes.small(n_points=300, width=16, height=16, spp=1)
    scenes.load_into(gpu_ctx, sc)
    gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    S = gpu_ctx.march_edges(want=True)[0]
    gpu_ctx.set_fw_schedule(4)  # the symmetric persistent solve, with its bounded waits
    try:
        dist = gpu_ctx.solve_paths(want=True)[0]
        ref = po.fw_minplus_f32(S)
        np.fill_diagonal(ref, 0.0)
        fin = np.isfinite(ref)
        assert np.array_equal(np.isfinite(dist), fin)
        assert np.allclose(dist[fin], ref[fin], rtol=1e-6, atol=0)
        # the solve's own error word is clear
        schedule, _ = gpu_ctx.fw_schedule()
        assert schedule == 4
    finally:
        gpu_ctx.set_fw_schedule(-1)
