"""LightGraph::outputDebugGeo (lg_geo_dump) and the command-line renderer's
reference flow (dart throwing, -geoDump) on the GPU. The dumped edges must be
the oracle's adjacency, the path weights its solved and column-normalised
transmittance, and the radiance the GPU's vertex data, each to the dump's six
significant digits."""
import os
import subprocess

import numpy as np
import pytest

from lightgraph_gb300 import build, scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def read(path):
    with open(path) as f:
        rows = [line.strip().split(",") for line in f if line.strip()]
    return np.array(rows, dtype=np.float64) if rows else np.zeros((0, 3))


def test_geo_dump_matches_oracle(gpu_ctx, tmp_path):
    sc = scenes.small(n_points=80, width=8, height=8, radius=0.3)
    scenes.load_into(gpu_ctx, sc)
    pts = sc.points[0]
    gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    gpu_ctx.solve_graphs(want=False)
    L, D = gpu_ctx.vertex_data()
    st = gpu_ctx.lib.lg_geo_dump(gpu_ctx.h, str(tmp_path).encode(), b"small", 7)
    assert st == 0, gpu_ctx.lib.lg_last_error(gpu_ctx.h)
    f = lambda k: os.path.join(tmp_path, f"small_{k}_0007.txt")
    assert np.allclose(read(f("pc")), pts, rtol=1e-5, atol=1e-7)
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)
    adj, _ = o.build_graph(pts, sc.radius_sq[0], sc.max_connect)
    iu = [(i, j) for i in range(len(pts)) for j in range(len(pts)) if i < j and adj[i, j]]
    edges = read(f("edge")).astype(int)
    assert [tuple(e) for e in edges] == iu
    T, _ = o.march_edges(pts, adj)
    Ts = o.fw_maxtimes(T)
    P = Ts / np.maximum(Ts.sum(axis=0, keepdims=True), 1.0)
    marching = read(f("marching"))
    ref = np.array([P[i, j] for i, j in iu])
    assert np.allclose(marching, ref, rtol=2e-4, atol=1e-7)
    assert np.allclose(read(f("light")), L.reshape(-1, 3), rtol=1e-5, atol=1e-9)
    assert np.allclose(read(f("diffuse")), D.reshape(-1, 3), rtol=1e-5, atol=1e-9)


def test_cli_reference_flow(tmp_path):
    exe = build.cli_path()
    out = tmp_path / "frame.exr"
    r = subprocess.run([exe, "-synthetic", "sphere:64", "-iter", "2", "-resWidth", "24", "-resHeight", "16",
                        "-light", "dir:0:1,1,1:1.0:-35,25,0", "-exrOut", str(out), "-geoDump", "-v"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.exists() and out.stat().st_size > 24 * 16 * 13 * 4
    for k in ("pc", "edge", "marching", "light", "diffuse"):
        for it in range(2):
            assert (tmp_path / "geoDump" / f"sphere_64_{k}_{it:04d}.txt").exists(), (k, it)
    n0 = len(read(tmp_path / "geoDump" / "sphere_64_pc_0000.txt"))
    assert 100 < n0 <= 751
