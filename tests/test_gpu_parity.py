"""GPU path vs the CPU oracle, stage by stage and end to end.

Tolerances (stated per test):
  adjacency            bit-exact
  Floyd-Warshall       <= 1e-6 relative vs the oracle's FP32 min-plus on the same input
  edge optical depth   <= 1e-4 relative vs FP64 (FP32 accumulation on the GPU)
  vertex light / D     <= 1e-4 relative vs FP64
  scatter grid         <= 1e-4 relative vs FP64 on the same radiances
  films (AOVs)         relative RMSE <= 1e-3 vs the FP64 oracle
"""
import numpy as np
import pytest

from lightgraph_gb300 import scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt(np.mean(b * b))
    if den == 0:
        return float(np.sqrt(np.mean(a * a)))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den)


def rand_graph_matrix(n, p, seed, symmetric=True):
    rng = np.random.default_rng(seed)
    S = np.full((n, n), np.inf, np.float32)
    mask = rng.random((n, n)) < p
    w = rng.random((n, n)).astype(np.float32) * 3.0
    S[mask] = w[mask]
    if symmetric:
        S = np.minimum(S, S.T)
    return S


@pytest.mark.parametrize("n", [1, 2, 5, 63, 64, 65, 127, 128, 129, 200, 333, 512])
def test_fw_matches_oracle_f32(gpu_ctx, n):
    S = rand_graph_matrix(n, min(1.0, 6.0 / max(n, 1)), seed=n)
    got = gpu_ctx.fw_host(S)
    ref = po.fw_minplus_f32(S)
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), fin)
    rel = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-30)
    assert rel.max(initial=0) <= 1e-6
    ref64 = po.fw_minplus_f64(S.astype(np.float64))
    rel64 = np.abs(got[fin] - ref64[fin]) / np.maximum(np.abs(ref64[fin]), 1e-30)
    assert rel64.max(initial=0) <= 1e-5


def test_fw_general_nonsymmetric(gpu_ctx):
    S = rand_graph_matrix(300, 0.03, seed=7, symmetric=False)
    got = gpu_ctx.fw_host(S)
    ref = po.fw_minplus_f32(S)
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), fin)
    assert np.allclose(got[fin], ref[fin], rtol=1e-6, atol=0)


@pytest.fixture(scope="module")
def small_scene():
    return scenes.small(n_points=512, width=64, height=64, spp=2)


@pytest.fixture(scope="module")
def small_oracle(small_scene):
    sc = small_scene
    return po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)


@pytest.mark.parametrize("max_connect", [0, 1, 3, 12, 16, 17])
@pytest.mark.parametrize("radius", [0.05, 0.15, 0.4])
def test_adjacency_bitexact(gpu_ctx, small_scene, max_connect, radius):
    sc = small_scene
    pts = sc.points[0]
    r2 = np.float32(radius) * np.float32(radius)
    adj, ne = gpu_ctx.build_graphs([pts], [r2], max_connect, want_adjacency=True)
    ref, ne_ref = po.build_graph(pts, r2, max_connect)
    assert np.array_equal(adj[0], ref)
    assert ne[0] == ne_ref


def test_adjacency_ties_and_many_graphs(gpu_ctx):
    rng = np.random.default_rng(3)
    graphs, r2s = [], []
    for g, n in enumerate([0, 1, 7, 100, 300, 257]):
        p = (rng.random((n, 3)).astype(np.float32) - 0.5) * 0.5
        if n > 10:
            p[5] = p[3]          # coincident points
            p[8] = p[3] + np.float32(0.1)  # exactly on a lattice offset
        graphs.append(p)
        r2s.append(np.float32(0.1) * np.float32(0.1))
    adj, ne = gpu_ctx.build_graphs(graphs, r2s, 12, want_adjacency=True)
    for g, p in enumerate(graphs):
        ref, ne_ref = po.build_graph(p, r2s[g], 12)
        assert np.array_equal(adj[g], ref), g
        assert ne[g] == ne_ref


def test_adjacency_dense_cluster_overflow(gpu_ctx):
    # more than the stored candidate capacity per row: the greedy pass must
    # continue the scan on the fly
    rng = np.random.default_rng(11)
    p = (rng.random((400, 3)).astype(np.float32) - 0.5) * 0.02
    r2 = np.float32(1.0)
    for mc in (12, 200):
        adj, ne = gpu_ctx.build_graphs([p], [r2], mc, want_adjacency=True)
        ref, ne_ref = po.build_graph(p, r2, mc)
        assert np.array_equal(adj[0], ref)


@pytest.fixture(scope="module")
def small_solved(gpu_ctx, small_scene, small_oracle):
    sc, o = small_scene, small_oracle
    scenes.load_into(gpu_ctx, sc)
    adj, _ = gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect, want_adjacency=True)
    S_gpu = gpu_ctx.march_edges(want=True)[0]
    dist_gpu = gpu_ctx.solve_paths(want=True)[0]
    L_gpu = gpu_ctx.vertex_light(want=True)
    D_gpu = gpu_ctx.diffuse(want=True)
    T, S_ref = o.march_edges(sc.points[0], adj[0])
    return dict(adj=adj[0], S_gpu=S_gpu, dist_gpu=dist_gpu, L_gpu=L_gpu, D_gpu=D_gpu, T=T, S_ref=S_ref)


def test_edge_march(small_solved):
    r = small_solved
    fin = np.isfinite(r["S_ref"])
    assert fin.sum() > 100
    assert np.array_equal(np.isfinite(r["S_gpu"]), fin)
    assert np.allclose(r["S_gpu"][fin], r["S_ref"][fin], rtol=1e-4, atol=1e-6)
    # the reference's RGB edge transmittance is exp(extinction_c * S)
    T = r["T"]
    nz = T[..., 0] > 0
    assert np.array_equal(nz, fin)
    assert np.allclose(T[fin][:, 0], np.exp(-np.float64(0.1) * r["S_ref"][fin]), rtol=1e-12)


def test_apsp_pipeline(small_solved):
    r = small_solved
    ref = po.fw_minplus_f64(r["S_ref"])
    np.fill_diagonal(ref, 0.0)
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(r["dist_gpu"]), fin)
    rel = np.abs(r["dist_gpu"][fin] - ref[fin]) / np.maximum(ref[fin], 1e-12)
    assert rel.max() <= 1e-4
    # the FW kernel itself on the GPU's own S: FP32 oracle within 1e-6
    ref32 = po.fw_minplus_f32(r["S_gpu"])
    np.fill_diagonal(ref32, 0.0)
    assert np.allclose(r["dist_gpu"][fin], ref32[fin], rtol=1e-6, atol=0)


def test_vertex_light(small_solved, small_scene, small_oracle):
    L_ref = small_oracle.vertex_light(small_scene.points[0])
    assert np.allclose(small_solved["L_gpu"], L_ref, rtol=1e-4, atol=1e-6)


def test_diffuse(small_solved, small_scene, small_oracle):
    o = small_oracle
    Tsol = o.fw_maxtimes(small_solved["T"])
    L_ref = o.vertex_light(small_scene.points[0])
    D_ref = o.diffuse(Tsol, L_ref)
    assert np.allclose(small_solved["D_gpu"], D_ref, rtol=1e-4, atol=1e-6)


def test_splat_and_render(gpu_ctx, small_scene, small_oracle, small_solved):
    sc, o = small_scene, small_oracle
    gpu_ctx.splat()
    lo, dims, sg = gpu_ctx.scatter_grid()
    lo_r, dims_r, sg_ref, _ = o.splat(sc.points[0], small_solved["D_gpu"].astype(np.float64))
    assert tuple(lo) == tuple(lo_r) and tuple(dims) == tuple(dims_r)
    assert np.allclose(sg, sg_ref, rtol=1e-4, atol=1e-6)
    films = gpu_ctx.render(sc.opts)
    ref = o.render((lo, dims, sg))
    for k, name in enumerate(["rgba", "direct", "scatter", "emission"]):
        got = getattr(films, name)
        e = rel_rmse(got, ref[k])
        assert e <= 1e-3, (name, e)


def test_full_frame_vs_fp64_oracle(gpu_ctx, small_scene, small_oracle):
    sc, o = small_scene, small_oracle
    scenes.load_into(gpu_ctx, sc)
    films = gpu_ctx.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
    # FP64 reference-faithful chain on the CPU
    adj, _ = o.build_graph(sc.points[0], sc.radius_sq[0], sc.max_connect)
    T, _ = o.march_edges(sc.points[0], adj)
    Tsol = o.fw_maxtimes(T)
    L = o.vertex_light(sc.points[0])
    D = o.diffuse(Tsol, L)
    lo, dims, sg, _ = o.splat(sc.points[0], D)
    ref = o.render((lo, dims, sg))
    for k, name in enumerate(["rgba", "direct", "scatter", "emission"]):
        e = rel_rmse(getattr(films, name), ref[k])
        assert e <= 1e-3, (name, e)


@pytest.mark.parametrize("wh", [(2, 2), (5, 3), (7, 2)])
def test_tiny_env_maps_vs_fp64_oracle(gpu_ctx, wh):
    """Environment maps at the smallest accepted size and with odd widths
    (the CDF guide tables cover fewer entries than guide points; edge texels
    wrap in the column and clamp in the row): the whole frame against the
    FP64 oracle, each AOV within 1e-3 rel-RMSE."""
    from lightgraph_gb300 import Light
    w, h = wh
    sc = scenes.small(n_points=200, width=24, height=24, spp=1)
    rng = np.random.default_rng(10 * w + h)
    env = (rng.random((h, w, 3)) * 4.0 + 0.1).astype(np.float32)
    sc.lights = list(sc.lights) + [Light.parse("env:0:1,1,1:0.5:2:sky")]
    sc.env_map = env
    scenes.load_into(gpu_ctx, sc)
    films = gpu_ctx.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights, env_map=env)
    adj, _ = o.build_graph(sc.points[0], sc.radius_sq[0], sc.max_connect)
    T, _ = o.march_edges(sc.points[0], adj)
    L = o.vertex_light(sc.points[0])
    D = o.diffuse(o.fw_maxtimes(T), L)
    lo, dims, sg, _ = o.splat(sc.points[0], D)
    ref = o.render((lo, dims, sg))
    for k, name in enumerate(["rgba", "direct", "scatter", "emission"]):
        e = rel_rmse(getattr(films, name), ref[k])
        assert e <= 1e-3, (wh, name, e)


def test_emission_telescopes_to_alpha(gpu_ctx):
    """The oracle's known answer on the GPU path: no lights, no scatter grid,
    a grey medium at a constant temperature. The emission AOV is the emission
    colour times the alpha in every pixel (the per-sample sum telescopes to
    1 - pTrans; FP32 accumulation: 1e-4), and every AOV matches the FP64
    oracle (rel-RMSE 1e-3)."""
    from lightgraph_gb300 import Context
    from lightgraph_gb300.lightgraph import ColorRamp, Grid, SceneSettings, Shader
    res = 32
    dens = np.zeros((res, res, res), np.float32)
    dens[8:24, 8:24, 8:24] = 0.6
    g = Grid(dens, (-16,) * 3, 0.05)
    temp = Grid(np.full((48, 48, 48), 700.0, np.float32), (-24,) * 3, 0.05)
    sh = Shader()
    sh.setScattering(0.3)
    sh.setAbsorption(0.1)
    sh.setEmissionScale(2.0)
    sh.setEmissionColorRamp(ColorRamp.parse("0,1/1,0.5,0.25:1,0.5,0.25/0/1000"))
    opts = SceneSettings(width=12, height=10, samples=2, camTranslate=(0, 0, 3), iter=1)
    ctx = Context(0)  # a fresh context: no scatter grid from earlier tests
    try:
        ctx.upload_density(g)
        ctx.upload_temperature(temp)
        ctx.set_shader(sh)
        ctx.set_settings(opts)
        ctx.set_lights([])
        films = ctx.render(opts)
    finally:
        ctx.close()
    alpha = films.rgba[..., 3].astype(np.float64)
    assert alpha.max() > 0.3 and alpha.min() == 0.0
    assert (films.direct == 0).all() and (films.scatter == 0).all()
    E = np.array([1.0, 0.5, 0.25]) * 2.0
    assert np.allclose(films.emission[..., :3], E * alpha[..., None], rtol=1e-4, atol=1e-4)
    ref = po.Oracle(g, sh, opts, [], temperature=temp).render()
    for got, r in ((films.rgba, ref[0]), (films.emission, ref[3])):
        assert rel_rmse(got, r) <= 1e-3


def test_vertex_light_unshadowed_known_answer():
    """The oracle's unshadowed known answer on the GPU path: in a medium
    thinner than the cutoff every shadow sample is skipped, so a vertex sees
    albedo * colour * intensity from a distant light and the same over
    1 + 4 pi r^2 from a point light (FP32: 1e-5)."""
    if not pytest.importorskip("torch").cuda.is_available():
        pytest.skip("no CUDA device")
    from lightgraph_gb300 import Context
    from lightgraph_gb300.lightgraph import Grid, Light, SceneSettings, Shader
    g = Grid(np.full((32, 32, 32), 1e-6, np.float32), (-16,) * 3, 1.0)
    sh = Shader()
    sh.setScattering(0.09)
    sh.setAbsorption(0.01)
    albedo = np.array(sh.getAlbedo())
    pts = np.array([[0.5, -3.25, 2.0], [-7.5, 6.0, -1.5], [10.25, 0.0, 4.75]], np.float32)
    pos = np.array([3.0, -2.0, 25.0])
    r2 = np.array([float(np.float32(np.sum((p.astype(np.float64) - pos) ** 2))) for p in pts])
    cases = [("dir:0:1,0.5,0.25:2.0:-40,30,0", np.tile(albedo * np.array([1.0, 0.5, 0.25]) * 2.0, (3, 1))),
             ("point:0:0.4,0.6,1.0:30:3,-2,25",
              albedo * np.array([0.4, 0.6, 1.0]) * 30.0 / (1.0 + 4.0 * np.pi * r2[:, None]))]
    ctx = Context(0)
    try:
        ctx.upload_density(g)
        ctx.upload_temperature(None)
        ctx.set_shader(sh)
        ctx.set_settings(SceneSettings(iter=1))
        ctx.build_graphs([pts], [np.float32(0.0)], 12)
        for spec, expect in cases:
            ctx.set_lights([Light.parse(spec)])
            L = ctx.vertex_light(want=True)
            assert np.allclose(L, expect, rtol=1e-5, atol=0), (spec, L, expect)
    finally:
        ctx.close()


def test_edge_march_density_min_known_answer():
    """The oracle's known answer on the GPU's edge march: inside existing
    leaves of zero density an edge gathers scatterDensityMin * step per sample
    while scatterDensityMin is at or above the cutoff, and nothing below it
    (src/LightGraph.h:390-395)."""
    if not pytest.importorskip("torch").cuda.is_available():
        pytest.skip("no CUDA device")
    from lightgraph_gb300 import Context
    from lightgraph_gb300.lightgraph import Grid, SceneSettings, Shader
    res = 32
    g = Grid(np.zeros((res, res, res), np.float32), (-res // 2,) * 3, 1.0,
             leaf_mask=np.ones((res // 8,) * 3, np.uint8))
    p = np.array([[-12.3, 0.2, 0.1], [11.7, 0.2, 0.1]], np.float32)
    dist = float(np.float32(np.linalg.norm(p[1].astype(np.float64) - p[0].astype(np.float64))))
    n_samples = len(np.arange(np.ceil(1e-9 / 3.0), np.floor(dist / 3.0) + 1))
    r2 = np.float32(30.0) * np.float32(30.0)
    ctx = Context(0)
    try:
        ctx.upload_density(g)
        ctx.upload_temperature(None)
        ctx.set_settings(SceneSettings(iter=1))
        for dmin, expect in ((0.025, n_samples * 0.025 * 3.0), (0.001, 0.0)):
            sh = Shader()
            sh.setScattering(0.09)
            sh.setAbsorption(0.01)
            sh.setScatterDensityMin(dmin)
            ctx.set_shader(sh)
            ctx.build_graphs([p], [r2], 12)
            S = ctx.march_edges(want=True)[0]
            assert S[0, 1] == S[1, 0]
            assert S[0, 1] == pytest.approx(expect, rel=1e-5, abs=1e-7), (dmin, S[0, 1], expect)
    finally:
        ctx.close()


def test_color_ramp_wrap_on_gpu():
    """ColorRamp::getColor's blend past the last knot (towards the first knot,
    with a negative weight) and between knots, through the GPU's vertex
    emission (no lights: L = ramp(temperature) * emissionScale), against the
    same known answers as the oracle's test (FP32: 1e-5)."""
    if not pytest.importorskip("torch").cuda.is_available():
        pytest.skip("no CUDA device")
    from lightgraph_gb300 import Context
    from lightgraph_gb300.lightgraph import ColorRamp, Grid, SceneSettings, Shader
    from .test_oracle import ramp_wrap_cases
    res = 32
    sh = Shader()
    sh.setEmissionScale(2.0)
    sh.setEmissionColorRamp(ColorRamp([0.2, 0.8], [[1, 0, 0], [0, 0, 1]], 100.0, 300.0))
    ctx = Context(0)
    try:
        ctx.upload_density(Grid(np.full((res, res, res), 0.5, np.float32), (-16,) * 3, 1.0))
        ctx.set_shader(sh)
        ctx.set_settings(SceneSettings(iter=1))
        ctx.set_lights([])
        ctx.build_graphs([np.zeros((1, 3), np.float32)], [np.float32(0.0)], 12)
        for temp, expect in ramp_wrap_cases():
            ctx.upload_temperature(Grid(np.full((res, res, res), temp, np.float32), (-16,) * 3, 1.0))
            L = ctx.vertex_light(want=True)
            assert np.allclose(L[0], 2.0 * expect, rtol=1e-5, atol=1e-6), (temp, L[0], expect)
    finally:
        ctx.close()


def test_deterministic(gpu_ctx, small_scene):
    sc = small_scene
    scenes.load_into(gpu_ctx, sc)
    a = gpu_ctx.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
    b = gpu_ctx.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
    for name in ["rgba", "direct", "scatter", "emission"]:
        assert np.array_equal(getattr(a, name), getattr(b, name))


def test_render_wave_times_after_lg_render(gpu_ctx, small_scene, small_solved):
    """Profiling covers a render made through lg_render as well as a frame:
    the five wave timers are positive and add up to less than the call."""
    import time
    sc = small_scene
    gpu_ctx.lib.lg_set_profiling(gpu_ctx.h, 1)
    try:
        gpu_ctx.splat()
        t0 = time.perf_counter()
        gpu_ctx.render(sc.opts)
        wall_ms = (time.perf_counter() - t0) * 1e3
        waves = gpu_ctx.render_wave_times()
    finally:
        gpu_ctx.lib.lg_set_profiling(gpu_ctx.h, 0)
    assert all(w > 0 for w in waves), waves
    assert sum(waves) < wall_ms


def test_grid_index_box_limit():
    """The marches take floors of index-space coordinates from float bits,
    exact below 2^22 voxels: a grid whose padded brick box (one brick of
    margin) reaches past +-(2^22 - 64) is refused, one just inside is taken."""
    from lightgraph_gb300 import Context, Grid, LightGraphError
    ctx = Context(0)
    try:
        vals = np.ones((8, 8, 8), np.float32)
        lim = 1 << 22
        for origin in [(lim - 128, 0, 0), (-lim + 128, 0, 0), (0, lim - 128, 0), (0, 0, -lim + 128)]:
            ctx.upload_density(Grid(vals, origin, 0.01))
        for origin in [(lim - 64, 0, 0), (-lim + 64, 0, 0), (0, lim, 0), (0, 0, -lim)]:
            with pytest.raises(LightGraphError):
                ctx.upload_density(Grid(vals, origin, 0.01))
    finally:
        ctx.close()


def test_expm1_approx_vs_library(gpu_ctx):
    """The primary wave's e^x - 1 (the Taylor series below |x| = 1/16,
    __expf(x) - 1 above) against the CUDA library's expm1f on the device,
    over the arguments its transmittance steps take (x <= 0, -extinction x
    density x step): relative error <= 4e-6."""
    from lightgraph_gb300 import _capi
    x = np.concatenate([-np.logspace(-10, np.log10(60.0), 40000),
                        [0.0, -0.0625, np.nextafter(np.float32(-0.0625), np.float32(0)),
                         np.nextafter(np.float32(-0.0625), np.float32(-1))]]).astype(np.float32)
    a = np.empty_like(x)
    r = np.empty_like(x)
    st = gpu_ctx.lib.lg_expm1_check(gpu_ctx.h, _capi.ptr(x), _capi.ptr(a), _capi.ptr(r), len(x))
    assert st == _capi.LG_OK
    ref = r.astype(np.float64)
    rel = np.abs(a.astype(np.float64) - ref) / np.maximum(np.abs(ref), 1e-38)
    assert rel.max() <= 4e-6, (float(rel.max()), float(x[np.argmax(rel)]))


def test_frame_after_failed_frame(small_scene):
    """A frame forks the render's count pass onto a side stream at its start;
    one that fails there (a zero-width camera) joins it again, and the next
    frame on the same context is bit-identical to one on a fresh context."""
    import copy
    from lightgraph_gb300 import Context, LightGraphError
    sc = small_scene
    bad = copy.deepcopy(sc.opts)
    bad.width = 0
    a = Context(0)
    b = Context(0)
    try:
        scenes.load_into(a, sc)
        scenes.load_into(b, sc)
        with pytest.raises(LightGraphError):
            a.render_frame(sc.points, sc.radius_sq, bad, sc.max_connect)
        fa = a.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
        fb = b.render_frame(sc.points, sc.radius_sq, sc.opts, sc.max_connect)
        for name in ["rgba", "direct", "scatter", "emission"]:
            assert np.array_equal(getattr(fa, name), getattr(fb, name)), name
    finally:
        a.close()
        b.close()
