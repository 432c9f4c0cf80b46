"""The point index's voxel size: points::computeVoxelSize(positions, 8) as
LightGraph::buildVdbPointGrid calls it (src/LightGraph.h:713-714). It sets the
splat kernel radius r = (3 K h^3 / (32 pi))^(1/3) (src/ScatterGrid.h:69-75).

Three restatements are compared: a pure-Python one here (small cases), the
oracle's (lgo_point_voxel_size) and the product's (lg_point_voxel_size, host
code of the CUDA library). The product's must equal the oracle's exactly on
the small (1024-point) and production (4096-point) point sets; no GPU needed."""
import math

import numpy as np
import pytest

from lightgraph_gb300 import _capi, scenes
from oracle import pyoracle as po


def voxel_size_py(pts, ppv=8):
    """OpenVDB's computeVoxelSize with an identity transform and five decimal
    places, written out loop by loop; float32 where OpenVDB stores floats."""
    f32 = np.float32
    n = len(pts)
    voxel = f32(0.1)
    if n <= 1:
        return float(voxel)
    target = max(1, n // ppv)
    p = [tuple(float(c) for c in q) for q in np.asarray(pts, np.float32)]
    lo = [min(q[a] for q in p) for a in range(3)]
    hi = [max(q[a] for q in p) for a in range(3)]
    if lo == hi:
        return float(voxel)
    ext = [hi[a] - lo[a] for a in range(3)]
    volume = ext[0] * ext[1] * ext[2]
    if abs(volume) <= 1e-15:
        e = sorted(ext)
        volume = e[2] ** 3 if abs(e[1]) <= 1e-15 else e[2] * e[1] * e[1]

    def from_volume(v):
        return f32(math.pow(v / target, 1.0 / 3.0))

    prev_volume = volume
    voxel = from_volume(volume)
    prev_count, count = 0, 1
    while count > prev_count:
        inv = 1.0 / float(voxel)
        cells = {tuple(math.floor(q[a] * inv + 0.5) for a in range(3)) for q in p}
        prev_count, count = count, len(cells)
        volume = float(f32(voxel * voxel * voxel) * f32(count))
        if volume >= prev_volume:
            break
        prev_volume = volume
        prev_voxel = voxel
        voxel = from_volume(volume)
        if f32(voxel / prev_voxel) > f32(0.9):
            break
    for d in range(5, 11):
        out = f32(math.floor(float(voxel) * 10.0 ** d + 0.5) / 10.0 ** d)
        if out != 0:
            return float(out)
    return float(voxel)


def product(pts):
    pts = np.ascontiguousarray(pts, np.float32)
    return _capi.load().lg_point_voxel_size(len(pts), pts.ctypes.data, 8)


def cases():
    rng = np.random.default_rng(5)
    out = {"empty": np.zeros((0, 3), np.float32), "one": np.ones((1, 3), np.float32),
           "coincident": np.full((20, 3), 0.25, np.float32)}
    for n in (2, 3, 7, 8, 9, 64, 300):
        out[f"box{n}"] = (rng.random((n, 3)) * [1.0, 0.5, 0.2] - 0.3).astype(np.float32)
    line = np.zeros((50, 3), np.float32)
    line[:, 1] = np.linspace(-1, 2, 50)
    out["collinear"] = line
    plane = np.zeros((80, 3), np.float32)
    plane[:, 0], plane[:, 2] = rng.random(80), rng.random(80) * 3
    out["coplanar"] = plane
    # two tight clusters: far fewer occupied voxels than the target, so the
    # refinement loop runs until the count stops growing
    cl = np.concatenate([rng.random((32, 3)) * 1e-3, 1.0 + rng.random((32, 3)) * 1e-3]).astype(np.float32)
    out["clusters"] = cl
    return out


@pytest.mark.parametrize("name", list(cases()))
def test_three_restatements_agree(name):
    pts = cases()[name]
    h_py = voxel_size_py(pts)
    assert po.point_voxel_size_of(pts) == h_py
    assert product(pts) == h_py


def test_clusters_refine_below_the_bbox_estimate():
    pts = cases()["clusters"]
    h = voxel_size_py(pts)
    bbox = np.prod(pts.max(0).astype(np.float64) - pts.min(0))
    estimate = (bbox / (len(pts) // 8)) ** (1 / 3)
    # two occupied voxels against a target of eight: the voxel shrinks twice
    assert h < 0.5 * estimate
    assert h == pytest.approx(estimate * 0.25 ** (2 / 3), rel=1e-3)


@pytest.mark.parametrize("which", ["small", "production"])
def test_product_equals_oracle_on_benchmark_points(which):
    sc = scenes.small() if which == "small" else scenes.production()
    pts = sc.points[0]
    h = po.point_voxel_size_of(pts)
    assert product(pts) == h
    # five decimal places, stored as a float
    assert np.float32(round(h, 5)) == np.float32(h)
    # the splat radius both sides derive from it (src/ScatterGrid.h:69-75)
    K = sc.opts.ptsPerKernel * sc.opts.iter
    r = ((3.0 * K * h ** 3) / (32.0 * math.pi)) ** (1.0 / 3.0)
    lo, dims, _, r_oracle = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights).splat(pts, np.zeros((len(pts), 3)))
    assert r_oracle == pytest.approx(r, rel=1e-14)
