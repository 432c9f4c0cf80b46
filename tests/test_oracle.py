"""Known-answer tests that pin the CPU oracle (the reference has no tests or
fixtures of its own, so these and tests/golden are the pins)."""
import numpy as np
import pytest

from lightgraph_gb300 import scenes
from lightgraph_gb300.lightgraph import ColorRamp, Grid, Light, SceneSettings, Shader
from oracle import pyoracle as po


def slab_scene(density=0.5, res=64):
    vals = np.full((res, res, res), density, np.float32)
    g = Grid(vals, (-res // 2,) * 3, 1.0)
    sh = Shader()
    sh.setScattering(0.09)
    sh.setAbsorption(0.01)
    opts = SceneSettings(width=8, height=8, iter=1)
    return g, sh, opts


def test_homogeneous_edge_transmittance():
    """Constant density: samples at t = k*step inside the span, each adding
    max(rho*dS*shadowDS*scatterDS, densityMin)*step."""
    g, sh, opts = slab_scene(0.5)
    o = po.Oracle(g, sh, opts)
    # two points along x, 30 voxels apart, well inside the grid
    p = np.array([[-15.3, 0.2, 0.1], [14.7, 0.2, 0.1]], np.float32)
    adj = np.array([[0, 1], [1, 0]], np.uint8)
    T, S = o.march_edges(p, adj)
    dist = float(np.linalg.norm(p[1].astype(np.float64) - p[0].astype(np.float64)))
    t0 = 1e-9  # Delta start time, inside the first leaf span
    ks = np.arange(np.ceil(t0 / 3.0), np.floor(np.float32(dist) / 3.0) + 1)
    x = max(0.5 * 1.0 * 1.0 * 0.35, 0.025)
    assert S[0, 1] == pytest.approx(len(ks) * x * 3.0, rel=1e-12)
    assert np.allclose(T[0, 1], np.exp(-0.1 * len(ks) * x * 3.0), rtol=1e-12)


def test_edge_march_density_min_in_empty_leaves():
    """Inside existing leaves of zero density an edge still gathers
    scatterDensityMin * step per sample while scatterDensityMin is at or above
    the cutoff (src/LightGraph.h:390-395), and nothing once it is below."""
    res = 32
    vals = np.zeros((res, res, res), np.float32)
    mask = np.ones((res // 8,) * 3, np.uint8)  # every leaf exists, all voxels 0
    g = Grid(vals, (-res // 2,) * 3, 1.0, leaf_mask=mask)
    sh = Shader()
    sh.setScattering(0.09)
    sh.setAbsorption(0.01)
    opts = SceneSettings(width=8, height=8, iter=1)
    p = np.array([[-12.3, 0.2, 0.1], [11.7, 0.2, 0.1]], np.float32)
    adj = np.array([[0, 1], [1, 0]], np.uint8)
    dist = float(np.float32(np.linalg.norm(p[1].astype(np.float64) - p[0].astype(np.float64))))
    ks = np.arange(np.ceil(1e-9 / 3.0), np.floor(dist / 3.0) + 1)
    T, S = po.Oracle(g, sh, opts).march_edges(p, adj)
    assert S[0, 1] == pytest.approx(len(ks) * 0.025 * 3.0, rel=1e-12)  # the default densityMin 0.025
    sh.setScatterDensityMin(0.001)  # below the cutoff 0.005: every sample skipped
    T, S = po.Oracle(g, sh, opts).march_edges(p, adj)
    assert S[0, 1] == 0.0 and np.allclose(T[0, 1], 1.0)


def test_edge_dropout_and_miss():
    g, sh, opts = slab_scene(1.0)
    sh.setScatterDensityScale(10.0)
    o = po.Oracle(g, sh, opts)
    p = np.array([[-25.0, 0, 0], [25.0, 0, 0], [0, 0, 1000.0]], np.float32)
    adj = np.ones((3, 3), np.uint8)
    np.fill_diagonal(adj, 0)
    T, S = o.march_edges(p, adj)
    assert np.isinf(S[0, 1]) and (T[0, 1] == 0).all()  # opaque: dropout
    assert S[0, 1] == S[1, 0]


def random_graph(n, p, seed):
    rng = np.random.default_rng(seed)
    S = np.full((n, n), np.inf)
    m = rng.random((n, n)) < p
    S[m] = rng.random((n, n))[m] * 2
    return np.minimum(S, S.T)


@pytest.mark.parametrize("n", [1, 7, 40, 150])
def test_fw_against_dijkstra(n):
    scipy = pytest.importorskip("scipy.sparse.csgraph")
    S = random_graph(n, 0.08, n)
    got = po.fw_minplus_f64(S)
    W = np.where(np.isfinite(S), S, 0.0)
    ref = scipy.dijkstra(W, directed=True)
    # FW keeps the (i, i) entries as shortest cycles; Dijkstra reports 0
    off = ~np.eye(n, dtype=bool)
    assert np.allclose(got[off], ref[off], rtol=1e-12)
    got32 = po.fw_minplus_f32(S.astype(np.float32))
    fin = np.isfinite(ref) & off
    assert np.allclose(got32[fin], ref[fin], rtol=1e-5)


def test_maxtimes_equals_minplus():
    """The reference's RGB max-times FW equals per-channel exp(-a_c * minplus(S))."""
    n = 60
    S = random_graph(n, 0.1, 3)
    a = np.array([0.1, 0.15, 0.3])
    T = np.where(np.isfinite(S)[..., None], np.exp(-a * np.where(np.isfinite(S), S, 0)[..., None]), 0.0)
    o = po.load()
    Tm = np.ascontiguousarray(T.copy())
    o.lgo_fw_maxtimes(n, Tm.ctypes.data)
    Sm = po.fw_minplus_f64(S)
    expect = np.where(np.isfinite(Sm)[..., None], np.exp(-a * np.where(np.isfinite(Sm), Sm, 0)[..., None]), 0.0)
    idx = np.arange(n)
    expect[idx, idx] = 1.0
    assert np.allclose(Tm, expect, rtol=1e-12, atol=1e-300)


def floyd_restated(T):
    """LightGraph::floydAlgo as the reference writes it (src/LightGraph.h:
    516-534): for k, for i with |T_ik|^2 > 0, for j with |T_kj|^2 > 0,
    T_ij = max per channel (T_ij, T_ik * T_kj), in place; then the diagonal is
    1. |v|^2 is the FP64 lengthSqr (x*x + y*y) + z*z, so a transmittance
    whose square underflows counts as no path."""
    T = T.copy()
    n = T.shape[0]

    def len2(v):
        return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]

    for k in range(n):
        for i in range(n):
            if len2(T[i, k]) > 0:
                for j in range(n):
                    if len2(T[k, j]) > 0:
                        T[i, j] = np.maximum(T[i, j], T[i, k] * T[k, j])
    for i in range(n):
        T[i, i] = 1.0
    return T


def test_floyd_against_the_reference_loop():
    """The oracle's max-times Floyd-Warshall equals floydAlgo's loop restated,
    bit for bit, on random symmetric RGB transmittance matrices, including
    entries so small that their squared length underflows (no path)."""
    rng = np.random.default_rng(23)
    o = po.Oracle(*slab_scene(0.5, res=16))
    for case in range(12):
        n = int(rng.integers(1, 18))
        T = rng.random((n, n, 3)) * (rng.random((n, n, 1)) < 0.35)
        if case % 4 == 3:
            T[rng.random((n, n)) < 0.2] = 1e-170  # |T|^2 underflows to 0
        T = np.maximum(T, T.transpose(1, 0, 2))
        for i in range(n):
            T[i, i] = 0.0
        assert np.array_equal(o.fw_maxtimes(T), floyd_restated(T)), case


def test_greedy_graph_cap_order():
    # five points on a line, all within the radius: the cap is spent in (i, j) order
    p = np.array([[0, 0, 0], [0.1, 0, 0], [0.2, 0, 0], [0.3, 0, 0], [0.4, 0, 0]], np.float32)
    adj, ne = po.build_graph(p, np.float32(1.0), max_connect=2)
    # i=0 takes 1 and 2 (full); i=1 skips 0 (full), takes 2 (1 and 2 now full);
    # i=2 is full; i=3 skips 0..2 (full) and takes 4.
    expect = np.zeros((5, 5), np.uint8)
    for i, j in [(0, 1), (0, 2), (1, 2), (3, 4)]:
        expect[i, j] = expect[j, i] = 1
    assert np.array_equal(adj, expect)
    assert ne == 4
    # strict radius: a pair exactly at the radius is not connected
    q = np.array([[0, 0, 0], [0.5, 0, 0]], np.float32)
    adj2, _ = po.build_graph(q, np.float32(0.25), 12)
    assert adj2.sum() == 0


def build_graph_restated(pts, r2, max_connect):
    """LightGraph::buildGraph's loop as the reference writes it
    (src/LightGraph.h:297-310): for i, for j, stop row i once it is full, skip
    a full j, connect i < j when the FP64 lengthSqr of the difference is below
    the FP32 radius squared."""
    n = len(pts)
    P = pts.astype(np.float64)
    cnt = [0] * n
    adj = np.zeros((n, n), np.uint8)
    edges = 0
    r2d = float(np.float32(r2))
    for i in range(n):
        for j in range(n):
            if cnt[i] >= max_connect:
                break
            if cnt[j] >= max_connect:
                continue
            if i < j:
                d = P[i] - P[j]
                if (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2] < r2d:
                    adj[i, j] = adj[j, i] = 1
                    cnt[i] += 1
                    cnt[j] += 1
                    edges += 1
    return adj, edges


def test_graph_build_against_the_reference_loop():
    """The oracle's graph build equals the reference's loop restated line by
    line, bit for bit, on random point sets: clustered and spread, radii that
    connect few or most pairs, caps from 0 to beyond any row's degree, and
    points on a lattice (exact ties at the radius)."""
    rng = np.random.default_rng(17)
    for case in range(60):
        n = int(rng.integers(1, 80))
        if case % 3 == 0:
            pts = (rng.integers(-3, 4, (n, 3)) * 0.25).astype(np.float32)  # lattice: exact distances
        elif case % 3 == 1:
            pts = (rng.normal(size=(n, 3)) * 0.1).astype(np.float32)
        else:
            pts = rng.random((n, 3)).astype(np.float32)
        r2 = np.float32(rng.choice([0.0625, 0.125, 0.25, 0.5]) ** 2 * (1 if case % 3 else 4))
        cap = int(rng.choice([0, 1, 2, 3, 12, 100]))
        adj, ne = po.build_graph(pts, r2, cap)
        ref, ne_ref = build_graph_restated(pts, r2, cap)
        assert np.array_equal(adj, ref), case
        assert ne == ne_ref, case


def test_color_ramp_knots_via_vertex_emission():
    res = 32
    vals = np.full((res, res, res), 0.5, np.float32)
    g = Grid(vals, (-16,) * 3, 1.0)
    sh = Shader()
    sh.setEmissionScale(2.0)
    sh.setEmissionColorRamp(ColorRamp([0.0, 0.5, 1.0], [[0, 0, 0], [1, 0.5, 0.25], [1, 1, 1]], 100.0, 300.0))
    opts = SceneSettings(iter=1)
    for temp, expect in [(100.0, [0, 0, 0]), (200.0, [1, 0.5, 0.25]), (300.0, [1, 1, 1]), (150.0, [0.5, 0.25, 0.125]),
                         (50.0, [0, 0, 0]), (1000.0, [1, 1, 1])]:
        tg = Grid(np.full((res, res, res), temp, np.float32), (-16,) * 3, 1.0)
        o = po.Oracle(g, sh, opts, [], temperature=tg)
        L = o.vertex_light(np.zeros((1, 3), np.float32))
        assert np.allclose(L[0], 2.0 * np.array(expect)), temp


def ramp_wrap_cases():
    """ColorRamp::getColor (src/Shader.h:63-92) with knots at 0.2 and 0.8 over
    temperatures 100..300: between the knots a linear blend; at a knot its
    colour; past the last knot the blend runs towards the FIRST knot (next
    stays at index 0), with a negative weight. Returns (temperature,
    expected colour) pairs."""
    pos, col = [0.2, 0.8], np.array([[1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    out = []
    for t in (200.0, 140.0, 260.0, 280.0, 300.0):
        x = min(max((t - 100.0) / (300.0 - 100.0), 0.0), 1.0)
        prev, nxt = 0, 0
        for i, p in enumerate(pos):
            if p <= x:
                prev = i
            else:
                nxt = i
                break
        b = (x - pos[prev]) / (pos[nxt] - pos[prev])
        out.append((t, col[prev] * (1.0 - b) + col[nxt] * b))
    return out


def test_color_ramp_wraps_past_the_last_knot():
    res = 32
    g = Grid(np.full((res, res, res), 0.5, np.float32), (-16,) * 3, 1.0)
    sh = Shader()
    sh.setEmissionScale(2.0)
    sh.setEmissionColorRamp(ColorRamp([0.2, 0.8], [[1, 0, 0], [0, 0, 1]], 100.0, 300.0))
    opts = SceneSettings(iter=1)
    cases = ramp_wrap_cases()
    assert np.allclose(cases[3][1], [-1.0 / 6.0, 0.0, 7.0 / 6.0])  # x = 0.9: weight -1/6 on the first knot
    for temp, expect in cases:
        tg = Grid(np.full((res, res, res), temp, np.float32), (-16,) * 3, 1.0)
        L = po.Oracle(g, sh, opts, [], temperature=tg).vertex_light(np.zeros((1, 3), np.float32))
        assert np.allclose(L[0], 2.0 * expect, rtol=1e-12, atol=1e-15), (temp, L[0], expect)


def ramp_restated(pos, col, t_in, t_out, t):
    """ColorRamp::getColor (src/Shader.h:56-92) line by line in FP64."""
    if len(pos) == 0:
        return np.zeros(3)
    x = min(max((t - t_in) / (t_out - t_in), 0.0), 1.0)
    if len(pos) == 1:
        return np.array(col[0], np.float64)
    prev = nxt = 0
    for i, p in enumerate(pos):
        if p <= x:
            prev = i
        else:
            nxt = i
            break
    rng_ = pos[nxt] - pos[prev]
    with np.errstate(divide="ignore", invalid="ignore"):
        b = (x - pos[prev]) / rng_ if rng_ != 0 else ((x - pos[prev]) * np.inf if x != pos[prev] else np.nan)
    return np.array(col[prev], np.float64) * (1.0 - b) + np.array(col[nxt], np.float64) * b


def test_color_ramp_against_the_reference_code():
    """The oracle's emission ramp equals getColor restated, bit for bit, on
    random ramps (1 to 5 sorted knots starting at 0, so no temperature falls
    below the first) and temperatures inside, at and past the range."""
    rng = np.random.default_rng(37)
    res = 16
    g = Grid(np.full((res, res, res), 0.5, np.float32), (-8,) * 3, 1.0)
    opts = SceneSettings(iter=1)
    for case in range(25):
        k = int(rng.integers(1, 6))
        pos = [0.0] + sorted(float(v) for v in rng.random(k - 1))
        col = [[float(c) for c in rng.random(3)] for _ in range(k)]
        sh = Shader()
        sh.setEmissionScale(1.0)
        sh.setEmissionColorRamp(ColorRamp(pos, col, 100.0, 900.0))
        for t in (float(np.float32(rng.uniform(0.0, 1200.0))), 100.0, 900.0, float(np.float32(100.0 + 800.0 * pos[-1]))):
            tg = Grid(np.full((res, res, res), t, np.float32), (-8,) * 3, 1.0)
            L = po.Oracle(g, sh, opts, [], temperature=tg).vertex_light(np.zeros((1, 3), np.float32))
            assert np.array_equal(L[0], ramp_restated(pos, col, 100.0, 900.0, t)), (case, t)


def test_env_cdf_step_function():
    """Distribution1D over a step function (src/Sampling.h:81-93): the CDF is
    the normalised running sum of func/n."""
    h, w = 4, 8
    env = np.zeros((h, w, 3), np.float32)
    env[:, 4:, :] = 1.0  # right half bright
    g, sh, opts = slab_scene(0.1, 16)
    o = po.Oracle(g, sh, opts, [Light.parse("env:0:1:1:2:x")], env_map=env)
    cf, cc, ci, mf, mc, mi = o.env_cdf()
    sin_t = np.sin(np.pi * (np.arange(h, dtype=np.float32) / np.float32(h - 1))).astype(np.float32)
    for r in range(h):
        if sin_t[r] == 0:
            assert np.allclose(cc[r], np.arange(w + 1) / w)
        else:
            assert np.allclose(cc[r], np.clip((np.arange(w + 1) - 4) / 4, 0, 1), atol=1e-7)
    assert mc[0] == 0 and mc[-1] == pytest.approx(1.0)


def splat_kernel(K, hp):
    """src/ScatterGrid.h:69-75: radius from the point index's voxel size
    (voxelSize^3 first, cube root by pow) and the truncated Gaussian's
    sigma^2 (weight 0.1 at the radius)."""
    r = ((3.0 * K * (hp * hp * hp)) / (32.0 * np.pi)) ** (1.0 / 3.0)
    return r, -(r * r) / (2.0 * np.log(0.1))


def voxel_d2(wpos, p):
    """Vec3s diff = worldPos - point, lengthSqr in float (ScatterGrid.h:86)."""
    e = [np.float32(wpos[a] - np.float64(p[a])) for a in range(3)]
    return np.float32(np.float32(e[0] * e[0] + e[1] * e[1]) + e[2] * e[2])


def test_splat_single_point_known_answer():
    """One point: every active coarse voxel whose centre lies within the
    kernel radius takes the point's radiance (a weighted mean of one value),
    every other voxel 0 (src/ScatterGrid.h:77-98)."""
    g, sh, opts = slab_scene(1.0, res=32)   # every coarse voxel active
    o = po.Oracle(g, sh, opts)
    pts = np.array([[1.3, -0.7, 2.1]], np.float32)
    D = np.array([[0.2, 0.5, 0.9]])
    K, hp, f = 3.0, 8.0, 4
    lo, dims, out, r = o.splat(pts, D, point_voxel_size=hp, factor=f, kernel_points=K)
    r_ref, _ = splat_kernel(K, hp)
    assert r == pytest.approx(r_ref, rel=1e-15)
    H = 1.0 * f
    inside = 0
    for cz in range(dims[2]):
        for cy in range(dims[1]):
            for cx in range(dims[0]):
                wpos = ((lo[0] + cx) * H, (lo[1] + cy) * H, (lo[2] + cz) * H)
                v = out[cz, cy, cx]
                if float(voxel_d2(wpos, pts[0])) < r_ref * r_ref:
                    inside += 1
                    assert np.allclose(v, D[0], rtol=1e-15, atol=0)
                else:
                    assert (v == 0).all()
    assert inside > 0


def test_splat_two_points_weighted_mean():
    """Two points around one coarse voxel: the Gaussian-weighted mean with
    w = exp(-d^2 / (2 sigma^2)) (src/ScatterGrid.h:84-95)."""
    g, sh, opts = slab_scene(1.0, res=32)
    o = po.Oracle(g, sh, opts)
    K, hp, f = 3.0, 8.0, 4
    r, s2 = splat_kernel(K, hp)
    H = 1.0 * f
    # points near the coarse voxel centred at the world origin
    pts = np.array([[0.9, 0.4, -0.3], [-1.7, 1.1, 0.6]], np.float32)
    D = np.array([[1.0, 0.0, 0.25], [0.0, 2.0, 0.75]])
    lo, dims, out, _ = o.splat(pts, D, point_voxel_size=hp, factor=f, kernel_points=K)
    c = [-lo[a] for a in range(3)]  # the coarse voxel at index 0 (world origin)
    w = [np.exp(-(1.0 / (2.0 * s2)) * float(voxel_d2((0.0, 0.0, 0.0), p))) for p in pts]
    assert all(float(voxel_d2((0.0, 0.0, 0.0), p)) < r * r for p in pts)
    expect = (D[0] * w[0] + D[1] * w[1]) / (w[0] + w[1])
    assert np.allclose(out[c[2], c[1], c[0]], expect, rtol=1e-12, atol=0)
    # the weight at exactly the radius is the truncation tail, 0.1
    assert np.exp(-(1.0 / (2.0 * s2)) * r * r) == pytest.approx(0.1, rel=1e-12)


def test_vertex_light_unshadowed_known_answer():
    """A medium thinner than the cutoff everywhere: every shadow sample is
    skipped (src/LightGraph.h:480), so each vertex sees the light unshadowed:
    albedo * I with I = colour * intensity for a distant light and
    colour * intensity / (1 + 4 pi r^2) for a point light, r^2 in float
    (src/Light.h:79-89,118-126)."""
    g, sh, opts = slab_scene(1e-6, res=32)
    albedo = np.array(sh.getAlbedo())
    pts = np.array([[0.5, -3.25, 2.0], [-7.5, 6.0, -1.5], [10.25, 0.0, 4.75]], np.float32)
    o = po.Oracle(g, sh, opts, [Light.parse("dir:0:1,0.5,0.25:2.0:-40,30,0")])
    L = o.vertex_light(pts)
    assert np.allclose(L, albedo * np.array([1.0, 0.5, 0.25]) * 2.0, rtol=1e-15, atol=0)
    pos = np.array([3.0, -2.0, 25.0])
    o = po.Oracle(g, sh, opts, [Light.parse("point:0:0.4,0.6,1.0:30:3,-2,25")])
    L = o.vertex_light(pts)
    for i, p in enumerate(pts):
        r2 = float(np.float32(np.sum((p.astype(np.float64) - pos) ** 2)))
        expect = albedo * np.array([0.4, 0.6, 1.0]) * 30.0 / (1.0 + 4.0 * np.pi * r2)
        assert np.allclose(L[i], expect, rtol=1e-12, atol=0), (i, L[i], expect)


def test_diffusion_known_answer():
    """diffuseLight (src/LightGraph.h:562-579): every column of the solved
    path matrix is divided by max(its sum, 1) per channel, then
    D_i = sum_j L_j * P_ij. With the diagonal at 1 (floydAlgo sets it,
    src/LightGraph.h:530-534) every column sums to at least 1; a matrix with a
    smaller diagonal shows the max(., 1): its thin columns are left as they
    are."""
    T = np.zeros((3, 3, 3))
    for i in range(3):
        T[i, i] = 1.0
    T[0, 1] = T[1, 0] = [0.5, 0.25, 0.125]
    T[1, 2] = T[2, 1] = [0.0, 0.5, 0.0]
    T[0, 2] = T[2, 0] = [0.25, 0.0, 0.75]
    L = np.array([[1.0, 2.0, 3.0], [0.5, 0.0, 1.0], [4.0, 1.0, 0.25]])
    o = po.Oracle(*slab_scene(0.5, res=16))
    D = o.diffuse(T, L)
    c = np.maximum(T.sum(axis=0), 1.0)       # per column j and channel
    expect = np.einsum("jc,ijc->ic", L, T / c[None, :, :])
    assert np.allclose(D, expect, rtol=1e-14, atol=0)
    assert c[2, 1] == 1.5  # 0 + 0.5 + 1
    # a diagonal of 0.25: column 1 sums to 0.25 + 0.5 + 0 = 0.75 in channel 0
    # (kept as it is), 0.25 + 0.25 + 0.5 = 1.0 in channel 1
    T2 = T.copy()
    for i in range(3):
        T2[i, i] = 0.25
    D2 = o.diffuse(T2, L)
    c2 = np.maximum(T2.sum(axis=0), 1.0)
    assert T2.sum(axis=0)[1, 0] == 0.75 and c2[1, 0] == 1.0
    assert np.allclose(D2, np.einsum("jc,ijc->ic", L, T2 / c2[None, :, :]), rtol=1e-14, atol=0)


def diffuse_restated(T, L):
    """LightGraph::diffuseLight as the reference writes it (src/LightGraph.h:
    562-579): column sums over i in order, maxComponent(sum, 1), the column
    divided by it, then D_i += L_j * P_ij over j in order."""
    P = T.copy()
    n = P.shape[0]
    for j in range(n):
        acc = np.zeros(3)
        for i in range(n):
            acc = acc + P[i, j]
        acc = np.maximum(acc, 1.0)
        for i in range(n):
            P[i, j] = P[i, j] / acc
    D = np.zeros((n, 3))
    for i in range(n):
        for j in range(n):
            D[i] = D[i] + L[j] * P[i, j]
    return D


def test_diffusion_against_the_reference_loop():
    """The oracle's diffusion equals diffuseLight's loops restated, bit for
    bit, on random solved path matrices and vertex radiance."""
    rng = np.random.default_rng(29)
    o = po.Oracle(*slab_scene(0.5, res=16))
    for case in range(10):
        n = int(rng.integers(1, 30))
        T = rng.random((n, n, 3)) * (rng.random((n, n, 1)) < 0.5)
        T = np.maximum(T, T.transpose(1, 0, 2))
        for i in range(n):
            T[i, i] = 1.0 if case % 2 == 0 else 0.3  # the solved diagonal, or a thin one
        L = rng.random((n, 3)) * 4.0
        assert np.array_equal(o.diffuse(T, L), diffuse_restated(T, L)), case


def test_splat_against_brute_force():
    """ScatterGrid::operator() (src/ScatterGrid.h:61-98) over every active
    coarse voxel with a brute-force search over all points: the oracle's cell
    search finds the same points (the same weighted means to rounding)."""
    g, sh, opts = slab_scene(1.0, res=32)
    o = po.Oracle(g, sh, opts)
    rng = np.random.default_rng(31)
    pts = ((rng.random((300, 3)) - 0.5) * 30.0).astype(np.float32)
    D = rng.random((300, 3))
    K, hp, f = 3.0, 6.0, 4
    lo, dims, out, r = o.splat(pts, D, point_voxel_size=hp, factor=f, kernel_points=K)
    r_ref, s2 = splat_kernel(K, hp)
    H = 1.0 * f
    P = pts.astype(np.float64)
    found = 0
    for cz in range(dims[2]):
        for cy in range(dims[1]):
            for cx in range(dims[0]):
                w = np.array([(lo[0] + cx) * H, (lo[1] + cy) * H, (lo[2] + cz) * H])
                e = (w[None, :] - P).astype(np.float32)
                d2 = (e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1]) + e[:, 2] * e[:, 2]   # float32, left to right
                near = d2.astype(np.float64) < r_ref * r_ref
                if near.any():
                    found += 1
                    wt = np.exp(-(1.0 / (2.0 * s2)) * d2[near].astype(np.float64))
                    expect = (D[near] * wt[:, None]).sum(0) / wt.sum()
                    assert np.allclose(out[cz, cy, cx], expect, rtol=1e-12, atol=0)
                else:
                    assert (out[cz, cy, cx] == 0).all()
    assert found > 50


def test_render_empty_grid_is_transparent():
    res = 16
    g = Grid(np.zeros((res, res, res), np.float32), (-8,) * 3, 0.1)
    sh = Shader()
    opts = SceneSettings(width=6, height=4, samples=2, camTranslate=(0, 0, 5), iter=1)
    o = po.Oracle(g, sh, opts, [Light.parse("dir:0:1:1:0,0,0")])
    rgba, direct, scatter, emission = o.render()
    assert np.all(rgba[..., :3] == 0) and np.all(rgba[..., 3] == 0)
    assert np.all(direct == 0) and np.all(scatter == 0) and np.all(emission == 0)


def test_render_emission_telescopes_to_alpha():
    """No lights and no scatter grid: the beauty is the emission AOV, and its
    per-sample sum of E * pTrans * (1 - dT), pTrans *= dT after each sample
    (src/Renderer.h:598,653-660), telescopes to E * (1 - pTrans at the end).
    With a grey extinction the alpha is 1 - pTrans (src/Renderer.h:674-677),
    so the emission AOV is the emission colour times the alpha in every
    pixel, whatever the jittered steps and early termination."""
    res = 32
    dens = np.zeros((res, res, res), np.float32)
    dens[8:24, 8:24, 8:24] = 0.6
    g = Grid(dens, (-16,) * 3, 0.05)
    # a constant temperature over a larger box: every sample reads 700
    temp = Grid(np.full((48, 48, 48), 700.0, np.float32), (-24,) * 3, 0.05)
    sh = Shader()
    sh.setScattering(0.3)
    sh.setAbsorption(0.1)
    sh.setEmissionScale(2.0)
    sh.setEmissionColorRamp(ColorRamp.parse("0,1/1,0.5,0.25:1,0.5,0.25/0/1000"))
    opts = SceneSettings(width=12, height=10, samples=2, camTranslate=(0, 0, 3), iter=1)
    o = po.Oracle(g, sh, opts, [], temperature=temp)
    rgba, direct, scatter, emission = o.render()
    alpha = rgba[..., 3]
    assert alpha.max() > 0.3 and alpha.min() == 0.0  # the cube and the background
    assert (direct == 0).all() and (scatter == 0).all()
    E = np.array([1.0, 0.5, 0.25]) * 2.0
    assert np.allclose(emission[..., :3], E * alpha[..., None], rtol=1e-9, atol=1e-15)
    assert np.allclose(rgba[..., :3], emission[..., :3], rtol=1e-15, atol=0)


def test_small_scene_oracle_runs_and_conserves_energy():
    sc = scenes.small(n_points=200, width=16, height=16)
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights)
    adj, ne = o.build_graph(sc.points[0], sc.radius_sq[0])
    assert ne > 100 and adj.sum(1).max() <= 12
    T, S = o.march_edges(sc.points[0], adj)
    Ts = o.fw_maxtimes(T)
    L = o.vertex_light(sc.points[0])
    D = o.diffuse(Ts, L)
    # column-normalised diffusion with all column sums >= 1 conserves total radiance
    colsum = Ts.sum(axis=0)
    if (colsum >= 1).all():
        assert np.allclose(D.sum(0), L.sum(0), rtol=1e-9)
