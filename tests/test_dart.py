"""Dart throwing (LightGraph::scatterPoints, src/LightGraph.h:206-274) on the CPU:
the host restatement of RandGen's mt19937 draws against the C++ library's
std::mt19937 / uniform_real_distribution<float> (through the oracle), the
C++ standard's known answer for mt19937, and properties of the oracle's
scatterPoints."""
import numpy as np
import pytest

from lightgraph_gb300 import lightgraph as lgm, scenes
from oracle import pyoracle as po


def test_mt19937_known_answer():
    # [rand.predef]: the 10000th output of a default-constructed mt19937 (seed 5489)
    _, raw = lgm.randgen_draws(5489, 10000)
    assert int(raw[9999]) == 4123659995


@pytest.mark.parametrize("seed", [5489, 854123, 854124, 854123 + 499])
def test_randgen_matches_std(seed):
    f, raw = lgm.randgen_draws(seed, 3 * 624 * 4 + 7)
    fo, rawo = po.randgen_draws(seed, len(f))
    assert np.array_equal(raw, rawo)
    assert np.array_equal(f.view(np.uint32), fo.view(np.uint32))
    assert f.min() >= 0.0 and f.max() < 1.0


def test_oracle_scatter_properties():
    sc = scenes.small(n_points=16)
    g = sc.density
    opts = lgm.scatter_opts(scatter_count=60000)
    pts, cnt, m2 = po.scatter_points(g, opts, 0, 2)
    pts2, cnt2, m22 = po.scatter_points(g, opts, 0, 2)
    assert np.array_equal(pts, pts2) and np.array_equal(cnt, cnt2) and np.array_equal(m2, m22)
    nz = np.argwhere(g.values != 0)  # z, y, x
    lo = (nz.min(0)[::-1] + np.array(g.origin)) * g.voxel_size
    hi = (nz.max(0)[::-1] + np.array(g.origin)) * g.voxel_size
    for i in range(2):
        assert 1 <= cnt[i] <= opts.target_size + 1
        p = pts[i, :cnt[i]]
        assert np.all(p >= lo - 1e-6) and np.all(p <= hi + 1e-6)
        d2 = ((p[:, None, :].astype(np.float64) - p[None, :, :]) ** 2).sum(-1)
        np.fill_diagonal(d2, np.inf)
        assert d2.min() > 0
        assert m2[i] > 0
    # different iterations use different engines
    assert not np.array_equal(pts[0, :cnt.min()], pts[1, :cnt.min()])
