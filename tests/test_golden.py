"""Committed golden vectors (tests/golden/*.npz, made by make_golden.py from the
oracle): the oracle must reproduce them, and the GPU path must match them
within the stated tolerances."""
import os

import numpy as np
import pytest

from tests.golden import make_golden as mg

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def rel_rmse(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = np.sqrt(np.mean(b * b))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else float(np.sqrt(np.mean(a * a)))


@pytest.mark.parametrize("name", mg.NAMES)
def test_oracle_reproduces_golden(name):
    g = load(name)
    now = mg.compute(name)
    assert np.array_equal(now["points"], g["points"])
    assert np.array_equal(now["adj"], g["adj"]) and int(now["n_edges"]) == int(g["n_edges"])
    for k in ["S", "T_solved", "S_solved", "L", "D"]:
        fin = np.isfinite(g[k])
        assert np.array_equal(np.isfinite(now[k]), fin), k
        assert np.allclose(now[k][fin], g[k][fin], rtol=1e-9, atol=1e-12), k
    assert np.allclose(now["scatter_grid"], g["scatter_grid"], rtol=1e-6, atol=1e-9)
    for k in ["rgba", "direct", "scatter", "emission"]:
        assert rel_rmse(now[k], g[k]) <= 1e-6, k


@pytest.mark.gpu
@pytest.mark.parametrize("name", mg.NAMES)
def test_gpu_matches_golden(gpu_ctx, name):
    from lightgraph_gb300 import scenes
    from oracle import pyoracle as po
    g = load(name)
    sc = mg.scene(name)
    scenes.load_into(gpu_ctx, sc)
    adj, ne = gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect, want_adjacency=True)
    assert np.array_equal(adj[0], g["adj"]) and int(ne[0]) == int(g["n_edges"])
    S = gpu_ctx.march_edges(want=True)[0]
    fin = np.isfinite(g["S"])
    assert np.array_equal(np.isfinite(S), fin)
    assert np.allclose(S[fin], g["S"][fin], rtol=1e-4, atol=1e-6)
    dist = gpu_ctx.solve_paths(want=True)[0]
    ref = g["S_solved"].copy()
    np.fill_diagonal(ref, 0.0)
    fin = np.isfinite(ref)
    assert np.allclose(dist[fin], ref[fin], rtol=1e-4, atol=1e-6)
    L = gpu_ctx.vertex_light(want=True)
    assert np.allclose(L, g["L"], rtol=1e-4, atol=1e-6)
    D = gpu_ctx.diffuse(want=True)
    assert np.allclose(D, g["D"], rtol=1e-4, atol=1e-6)
    gpu_ctx.splat()
    lo, dims, sg = gpu_ctx.scatter_grid()
    assert tuple(lo) == tuple(g["sg_lo"]) and tuple(dims) == tuple(g["sg_dims"])
    assert np.allclose(sg, g["scatter_grid"], rtol=1e-3, atol=1e-5)
    films = gpu_ctx.render(sc.opts)
    for k in ["rgba", "direct", "scatter", "emission"]:
        assert rel_rmse(getattr(films, k), g[k]) <= 1e-3, k
