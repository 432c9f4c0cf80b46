"""GPU dart throwing (lg_scatter_points / lg_scatter_graphs) against the
oracle's scatterPoints, which runs the C++ library's std::mt19937 as the
reference's RandGen does: the accepted point sets must be identical (same
points, bit for bit, in the same order) and so must the connect radii."""
import numpy as np
import pytest

from lightgraph_gb300 import lightgraph as lgm, scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def connect_r2(m2, mult):
    r = np.sqrt(np.float32(m2)) * np.float32(mult)
    return np.float32(r * r)


def check_iterations(ctx, sc, opts, first, n):
    pts, r2 = ctx.scatter_points(first, n, opts)
    opt, ocnt, om2 = po.scatter_points(sc.density, opts, first, n)
    for i in range(n):
        assert len(pts[i]) == ocnt[i], (first + i, len(pts[i]), ocnt[i])
        assert np.array_equal(pts[i].view(np.uint32), opt[i, :ocnt[i]].view(np.uint32)), first + i
        assert np.float32(r2[i]) == connect_r2(om2[i], opts.connect_mult), first + i
    return pts, r2


def test_scatter_points_match_oracle(gpu_ctx):
    sc = scenes.small(n_points=16)
    scenes.load_into(gpu_ctx, sc)
    opts = lgm.scatter_opts(scatter_count=200000)
    check_iterations(gpu_ctx, sc, opts, 0, 4)
    check_iterations(gpu_ctx, sc, opts, 37, 2)


def test_scatter_points_reference_constants(gpu_ctx):
    sc = scenes.small(n_points=16)
    scenes.load_into(gpu_ctx, sc)
    opts = lgm.scatter_opts()
    assert opts.scatter_count == 1000000 and opts.target_size == 750
    pts, _ = check_iterations(gpu_ctx, sc, opts, 0, 1)
    assert 100 < len(pts[0]) <= 751


def test_scatter_graphs_connects_like_oracle(gpu_ctx):
    sc = scenes.small(n_points=16)
    scenes.load_into(gpu_ctx, sc)
    opts = lgm.scatter_opts(scatter_count=150000)
    pts, r2 = gpu_ctx.scatter_points(0, 2, opts)
    cnt = gpu_ctx.scatter_graphs(0, 2, 12, opts)
    assert [len(p) for p in pts] == list(cnt)
    S_dev = gpu_ctx.march_edges(want=True)
    adj, _ = gpu_ctx.build_graphs(pts, r2, 12, want_adjacency=True)
    S_host = gpu_ctx.march_edges(want=True)
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)
    for i in range(2):
        assert np.array_equal(S_dev[i], S_host[i])
        oadj, ne = o.build_graph(pts[i], float(r2[i]), 12)
        assert ne > 0
        assert np.array_equal(adj[i].astype(bool), oadj.astype(bool))
