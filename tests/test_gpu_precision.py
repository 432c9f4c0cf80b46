"""Reduced-precision grid storage: density (and temperature) bricks stored as
FP16 or BF16, optical depth and transmittance accumulated in FP32, on the
small configuration (128^3 sphere-fBm, 1024 points, 256^2 at 1 spp) with the
512x256 sky map added as an importance-sampled environment light.

Parity: the GPU with FP16/BF16 bricks matches the FP64 oracle run on the same
quantised voxel values (rel. RMSE <= 1e-3 per AOV, distances <= 1e-4). The
error of the reduced storage itself -- the GPU on FP16/BF16 bricks against
the FP64 oracle on the FP32 grid -- is printed (PRECISION lines) and held to
the same 1e-3 per AOV."""
import numpy as np
import pytest
import torch

from lightgraph_gb300 import _capi, scenes
from lightgraph_gb300.lightgraph import Grid
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

DTYPES = {"fp16": (_capi.LG_DTYPE_F16, torch.float16), "bf16": (_capi.LG_DTYPE_BF16, torch.bfloat16)}


def rel_rmse(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = np.sqrt(np.mean(b * b))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else float(np.sqrt(np.mean(a * a)))


def quantise(vals, tdtype):
    return torch.from_numpy(vals).to(tdtype).to(torch.float32).numpy()


def oracle_frame(sc, dens_grid):
    o = po.Oracle(dens_grid, sc.shader, sc.opts, sc.lights, env_map=sc.env_map)
    pts = sc.points[0]
    adj, _ = o.build_graph(pts, sc.radius_sq[0], sc.max_connect)
    T, S = o.march_edges(pts, adj)
    Tsol = o.fw_maxtimes(T)
    Smin = po.fw_minplus_f64(S)
    L = o.vertex_light(pts)
    D = o.diffuse(Tsol, L)
    lo, dims, sg, _ = o.splat(pts, D)
    return Smin, D, o.render((lo, dims, sg))


@pytest.mark.parametrize("name", ["fp16", "bf16"])
def test_reduced_precision_bricks(gpu_ctx, name):
    code, tdtype = DTYPES[name]
    sc = scenes.with_envmap(scenes.small())
    assert sc.env_map.shape == (256, 512, 3)
    scenes.load_into(gpu_ctx, sc, dtype=code)
    films = gpu_ctx.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
    dist = gpu_ctx.solve_paths(want=True)[0]
    g = sc.density
    q = Grid(quantise(g.values, tdtype), g.origin, g.voxel_size)
    S_q, D_q, ref_q = oracle_frame(sc, q)
    S_f, D_f, ref_f = oracle_frame(sc, g)
    # parity against the oracle on the same stored values
    for k, film in enumerate(["rgba", "direct", "scatter", "emission"]):
        assert rel_rmse(getattr(films, film), ref_q[k]) <= 1e-3, (name, film)
    fin = np.isfinite(S_q)
    np.fill_diagonal(S_q, 0.0)
    both = fin & np.isfinite(dist)
    dist_rel_q = float(np.max(np.abs(dist[both] - S_q[both]) / np.maximum(S_q[both], 1e-12)))
    assert dist_rel_q <= 1e-4
    # the storage error itself, against FP64 on the FP32 grid
    errs = {film: rel_rmse(getattr(films, film), ref_f[k])
            for k, film in enumerate(["rgba", "direct", "scatter", "emission"])}
    np.fill_diagonal(S_f, 0.0)
    both = np.isfinite(S_f) & np.isfinite(dist)
    dist_rel = float(np.median(np.abs(dist[both] - S_f[both]) / np.maximum(S_f[both], 1e-12)))
    reach_diff = int((np.isfinite(S_f) != np.isfinite(dist)).sum())
    print(f"PRECISION {name} " + " ".join(f"{k}={v:.2e}" for k, v in errs.items()) +
          f" dist_median_rel={dist_rel:.2e} reachability_differs={reach_diff}")
    for film, e in errs.items():
        assert e <= 1e-3, (name, film, e)
