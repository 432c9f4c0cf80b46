"""Parity at the benchmark configurations themselves, against the FP64 oracle.

  small (128^3 dense sphere-fBm, 1024 points, radius 0.15, 256^2 at 1 spp):
      the whole frame end to end, every stage and all four AOVs.
  production (512^3 sparse cumulus, 4096 points, 1024^2 at 4 spp, a distant
      and a point light, temperature through a ramp):
      adjacency bit-exact at N = 4096; edge optical depth; the whole 4096^2
      distance matrix against the oracle's FP32 min-plus on the same input;
      rows from 16 sources against FP64 Dijkstra on the oracle's own edges;
      vertex light and diffusion; a band of 8 image rows spread over the
      frame against the oracle's render of those rows.
  batched (64 graphs, N log-uniform in [256, 4096], seed 3, one persistent
      Floyd-Warshall launch): every graph against the oracle.
  reference-style multi-iteration frame (6 dart-thrown LightGraphs in the
      small volume, one splat with K = ptsPerKernel * iter): whole frame.

Tolerances (as elsewhere): adjacency bit-exact; distances <= 1e-6 relative to
the oracle's FP32 min-plus on the same edge weights and <= 1e-4 relative to
FP64 on the oracle's own edge weights (FP32 accumulation along an edge);
edge optical depth, vertex light and diffusion <= 1e-4 relative; each AOV
relative RMSE <= 1e-3. The production frame's oracle uses FP64 Dijkstra for
the all-pairs solve (the min-plus form of floydAlgo's max-times loop)."""
import numpy as np
import pytest

from lightgraph_gb300 import lightgraph as lgm, scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

AOVS = ["rgba", "direct", "scatter", "emission"]


def rel_rmse(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = np.sqrt(np.mean(b * b))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else float(np.sqrt(np.mean(a * a)))


def max_rel(got, ref):
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), fin)
    if not fin.any():
        return 0.0
    return float(np.max(np.abs(got[fin].astype(np.float64) - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-12)))


def oracle_chain(o, sc, pts_list, apsp="fw"):
    """The reference's LightGraph stage on the CPU for each graph, then one
    splat of every graph's points with the oracle's own point voxel size."""
    D_all, S_all, L_all = [], [], []
    for g, pts in enumerate(pts_list):
        adj, _ = o.build_graph(pts, sc.radius_sq[g], sc.max_connect)
        T, S = o.march_edges(pts, adj, want_T=(apsp == "fw"))
        Tsol = o.fw_maxtimes(T) if apsp == "fw" else po.transmittance_of(po.apsp_dijkstra_f64(S),
                                                                        sc.shader.getExtinction())
        L = o.vertex_light(pts, graph_id=g)
        D_all.append(o.diffuse(Tsol, L))
        S_all.append(S)
        L_all.append(L)
    pts = np.concatenate(pts_list)
    lo, dims, sg, _ = o.splat(pts, np.concatenate(D_all))
    return (lo, dims, sg), S_all, L_all, D_all


# ---------------------------------------------------------------------------
# small: the whole frame as configured
# ---------------------------------------------------------------------------

def test_small_config_whole_frame(gpu_ctx):
    sc = scenes.small()
    assert (len(sc.points[0]), sc.opts.width, sc.opts.height, sc.opts.samples) == (1024, 256, 256, 1)
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)
    scenes.load_into(gpu_ctx, sc)
    adj, ne = gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect, want_adjacency=True)
    S = gpu_ctx.march_edges(want=True)[0]
    dist = gpu_ctx.solve_paths(want=True)[0]
    L = gpu_ctx.vertex_light(want=True)
    D = gpu_ctx.diffuse(want=True)
    gpu_ctx.splat()
    lo, dims, sg = gpu_ctx.scatter_grid()
    films = gpu_ctx.render(sc.opts)

    sg_ref, S_ref, L_ref, D_ref = oracle_chain(o, sc, sc.points)
    adj_ref, ne_ref = o.build_graph(sc.points[0], sc.radius_sq[0], sc.max_connect)
    assert np.array_equal(adj[0], adj_ref) and ne[0] == ne_ref
    assert max_rel(S, S_ref[0]) <= 1e-4
    ref32 = po.fw_minplus_f32(S)
    np.fill_diagonal(ref32, 0.0)
    assert max_rel(dist, ref32) <= 1e-6
    ref64 = po.fw_minplus_f64(S_ref[0])
    np.fill_diagonal(ref64, 0.0)
    assert max_rel(dist, ref64) <= 1e-4
    assert np.allclose(L, L_ref[0], rtol=1e-4, atol=1e-7)
    assert np.allclose(D, D_ref[0], rtol=1e-4, atol=1e-7)
    assert tuple(lo) == tuple(sg_ref[0]) and tuple(dims) == tuple(sg_ref[1])
    assert np.allclose(sg, sg_ref[2], rtol=1e-3, atol=1e-6)
    ref = o.render(sg_ref)
    errs = {k: rel_rmse(getattr(films, k), ref[i]) for i, k in enumerate(AOVS)}
    print("SMALL_CONFIG " + " ".join(f"{k}={v:.2e}" for k, v in errs.items()))
    for k, e in errs.items():
        assert e <= 1e-3, (k, e)
    # and the same frame through the one-call entry point
    scenes.load_into(gpu_ctx, sc)
    again = gpu_ctx.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
    for k in AOVS:
        assert np.array_equal(getattr(again, k), getattr(films, k)), k


# ---------------------------------------------------------------------------
# production: N = 4096, 1024^2 at 4 spp
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def production():
    sc = scenes.production()
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights, temperature=sc.temperature)
    return sc, o


@pytest.fixture(scope="module")
def production_gpu(gpu_ctx, production):
    sc, _ = production
    scenes.load_into(gpu_ctx, sc)
    adj, ne = gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect, want_adjacency=True)
    out = dict(adj=adj[0], ne=int(ne[0]), S=gpu_ctx.march_edges(want=True)[0],
               dist=gpu_ctx.solve_paths(want=True)[0], L=gpu_ctx.vertex_light(want=True),
               D=gpu_ctx.diffuse(want=True))
    gpu_ctx.splat()
    out["sg"] = gpu_ctx.scatter_grid()
    out["films"] = gpu_ctx.render(sc.opts)
    return out


@pytest.fixture(scope="module")
def production_oracle(production):
    sc, o = production
    pts = sc.points[0]
    adj, ne = o.build_graph(pts, sc.radius_sq[0], sc.max_connect)
    _, S = o.march_edges(pts, adj, want_T=False)
    apsp = po.apsp_dijkstra_f64(S)
    L = o.vertex_light(pts)
    D = o.diffuse(po.transmittance_of(apsp, sc.shader.getExtinction()), L)
    lo, dims, sg, _ = o.splat(pts, D)
    return dict(adj=adj, ne=int(ne), S=S, apsp=apsp, L=L, D=D, sg=(lo, dims, sg))


def test_production_adjacency_and_edges(production_gpu, production_oracle):
    g, r = production_gpu, production_oracle
    assert g["adj"].shape == (4096, 4096)
    assert np.array_equal(g["adj"], r["adj"]) and g["ne"] == r["ne"]
    assert max_rel(g["S"], r["S"]) <= 1e-4


def test_production_distances(production_gpu, production_oracle):
    g, r = production_gpu, production_oracle
    dist = g["dist"]
    # the whole matrix against the FP32 min-plus oracle on the same input
    ref32 = po.fw_minplus_f32(g["S"])
    np.fill_diagonal(ref32, 0.0)
    assert max_rel(dist, ref32) <= 1e-6
    # 16 spread sources against FP64 Dijkstra on the oracle's own edges
    src = np.linspace(0, 4095, 16).astype(int)
    assert max_rel(dist[src], r["apsp"][src]) <= 1e-4
    print(f"PRODUCTION_DIST vs_fp32={max_rel(dist, ref32):.2e} vs_fp64_rows={max_rel(dist[src], r['apsp'][src]):.2e}")


def test_production_light_and_diffusion(production_gpu, production_oracle):
    g, r = production_gpu, production_oracle
    assert np.allclose(g["L"], r["L"], rtol=1e-4, atol=1e-7)
    assert np.allclose(g["D"], r["D"], rtol=1e-4, atol=1e-7)


def test_production_image_rows(production, production_gpu, production_oracle):
    sc, o = production
    lo, dims, _ = production_gpu["sg"]
    assert tuple(lo) == tuple(production_oracle["sg"][0]) and tuple(dims) == tuple(production_oracle["sg"][1])
    H = sc.opts.height
    rows = [int((k + 0.5) * H / 8) for k in range(8)]
    ref = o.render(production_oracle["sg"], rows=rows)
    films = production_gpu["films"]
    errs = {}
    for i, k in enumerate(AOVS):
        got = getattr(films, k)[rows]
        errs[k] = rel_rmse(got, ref[i][rows])
    print("PRODUCTION_ROWS " + " ".join(f"{k}={v:.2e}" for k, v in errs.items()))
    assert np.abs(ref[0][rows][..., 3]).max() > 0.1  # the band crosses the cloud
    for k, e in errs.items():
        assert e <= 1e-3, (k, e)


# ---------------------------------------------------------------------------
# batched: 64 graphs of 256..4096 points in one persistent launch
# ---------------------------------------------------------------------------

def test_batched_config_every_graph(gpu_ctx):
    sc = scenes.batched_graphs()
    sizes = [len(p) for p in sc.points]
    assert len(sizes) == 64 and min(sizes) >= 256 and max(sizes) <= 4096
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)
    scenes.load_into(gpu_ctx, sc)
    adj, ne = gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect, want_adjacency=True)
    S = gpu_ctx.march_edges(want=True)
    gpu_ctx.set_fw_schedule(-1)
    dist = gpu_ctx.solve_paths(want=True)
    L = gpu_ctx.vertex_light(want=True)
    D = gpu_ctx.diffuse(want=True)
    off = np.concatenate([[0], np.cumsum(sizes)])
    worst = {"S": 0.0, "fp32": 0.0, "fp64": 0.0}
    for gi, pts in enumerate(sc.points):
        n = len(pts)
        a_ref, ne_ref = o.build_graph(pts, sc.radius_sq[gi], sc.max_connect)
        assert np.array_equal(adj[gi], a_ref) and ne[gi] == ne_ref, gi
        _, S_ref = o.march_edges(pts, a_ref, want_T=False)
        worst["S"] = max(worst["S"], max_rel(S[gi], S_ref))
        if n <= 1024:
            ref32 = po.fw_minplus_f32(S[gi])
            np.fill_diagonal(ref32, 0.0)
            worst["fp32"] = max(worst["fp32"], max_rel(dist[gi], ref32))
            src = None
        else:
            src = np.linspace(0, n - 1, 16).astype(int)
            # exact FP64 paths over the GPU's own FP32 edge weights: the FP32
            # sums along a path of <= n edges stay within 1e-5
            ref_own = po.apsp_dijkstra_f64(S[gi], src)
            worst["fp32"] = max(worst["fp32"], max_rel(dist[gi][src], ref_own) / 10.0)
        apsp = po.apsp_dijkstra_f64(S_ref)
        rows = slice(None) if src is None else src
        worst["fp64"] = max(worst["fp64"], max_rel(dist[gi][rows], apsp[rows]))
        L_ref = o.vertex_light(pts, graph_id=gi)
        D_ref = o.diffuse(po.transmittance_of(apsp, sc.shader.getExtinction()), L_ref)
        sl = slice(off[gi], off[gi + 1])
        assert np.allclose(L[sl], L_ref, rtol=1e-4, atol=1e-7), gi
        assert np.allclose(D[sl], D_ref, rtol=1e-4, atol=1e-7), gi
    print("BATCHED " + " ".join(f"{k}={v:.2e}" for k, v in worst.items()))
    assert worst["S"] <= 1e-4 and worst["fp32"] <= 1e-6 and worst["fp64"] <= 1e-4


# ---------------------------------------------------------------------------
# the reference's multi-iteration frame: dart-thrown graphs, one splat
# ---------------------------------------------------------------------------

def test_multi_iteration_frame(gpu_ctx):
    iters = 6
    sc = scenes.small(n_points=16, width=96, height=96, spp=2)
    sc.opts.iter = iters
    sc.opts.ptsPerKernel = 3
    opts = lgm.scatter_opts()
    scenes.load_into(gpu_ctx, sc)
    cnt = gpu_ctx.scatter_graphs(0, iters, sc.max_connect, opts)
    assert len(cnt) == iters and min(cnt) >= 200 and max(cnt) <= 751
    gpu_ctx.solve_graphs(want=False)
    gpu_ctx.splat()
    films = gpu_ctx.render(sc.opts)

    # the oracle's own dart throwing (the same points, bit for bit) and chain
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)
    opt, ocnt, om2 = po.scatter_points(sc.density, opts, 0, iters)
    assert list(ocnt) == list(cnt)
    pts = [opt[i, :ocnt[i]] for i in range(iters)]
    r = np.sqrt(om2.astype(np.float32)) * np.float32(opts.connect_mult)
    sc.radius = [float(x) for x in r]  # radius_sq recomputes r * r in float32
    sg, _, _, _ = oracle_chain(o, sc, pts)
    ref = o.render(sg)
    errs = {k: rel_rmse(getattr(films, k), ref[i]) for i, k in enumerate(AOVS)}
    print(f"MULTI_ITERATION points={sum(cnt)} " + " ".join(f"{k}={v:.2e}" for k, v in errs.items()))
    for k, e in errs.items():
        assert e <= 1e-3, (k, e)
