"""Many graphs of uneven size: the persistent batched Floyd-Warshall, its
autotuner, and frame replay through a captured CUDA graph."""
import numpy as np
import pytest

from lightgraph_gb300 import LightGraphError, _capi, scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def uneven_graphs():
    """12 graphs, sizes log-uniform in [20, 700] (seed 3), points inside the
    small scene's volume, connection radius 0.15."""
    sc = scenes.small(n_points=16, width=32, height=32)
    rng = np.random.default_rng(3)
    sizes = np.exp(rng.uniform(np.log(20), np.log(700), 12)).astype(int)
    pts = [scenes.points(sc.density.values, sc.density.voxel_size, int(n), seed=100 + g)
           for g, n in enumerate(sizes)]
    sc.points = pts
    sc.radius = [0.15] * len(pts)
    sc.opts.iter = len(pts)
    return sc


def solve_with(ctx, sc, schedule):
    scenes.load_into(ctx, sc)
    ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    S = ctx.march_edges(want=True)
    ctx.set_fw_schedule(schedule)
    dist = ctx.solve_paths(want=True)
    used, ms = ctx.fw_schedule()
    return S, dist, used, ms


def test_schedules_bit_identical_and_match_oracle(gpu_ctx, uneven_graphs):
    """Every schedule, the symmetric ones (3, 4, and 5 with its TMA-staged
    update operands) included, gives the same bits;
    the graphs up to 700 points run 12 rounds, so the symmetric solve reuses
    each of its three column-panel slots several times."""
    sc = uneven_graphs
    S0, d0, u0, _ = solve_with(gpu_ctx, sc, 0)
    assert u0 == 0
    for schedule in (1, 2, 3, 4, 5):
        _, ds, us, _ = solve_with(gpu_ctx, sc, schedule)
        assert us == schedule
        for g in range(len(sc.points)):
            assert np.array_equal(d0[g], ds[g]), (schedule, g)
    for g in range(len(sc.points)):
        assert np.array_equal(S0[g], S0[g].T), g  # the solve's symmetric input
        assert np.array_equal(d0[g], d0[g].T), g
        ref = po.fw_minplus_f32(S0[g])
        np.fill_diagonal(ref, 0.0)
        fin = np.isfinite(ref)
        assert np.array_equal(np.isfinite(d0[g]), fin)
        assert np.allclose(d0[g][fin], ref[fin], rtol=1e-6, atol=0), g


def test_fw_schedule_range(gpu_ctx, uneven_graphs):
    """Schedules -1..5 are accepted; anything else is LG_ERR_INVALID and
    leaves the schedule in force."""
    _, _, used, _ = solve_with(gpu_ctx, uneven_graphs, 5)
    assert used == 5
    for bad in (-2, 6):
        with pytest.raises(LightGraphError) as e:
            gpu_ctx.set_fw_schedule(bad)
        assert e.value.status == _capi.LG_ERR_INVALID
        assert gpu_ctx.fw_schedule()[0] == 5
    gpu_ctx.set_fw_schedule(-1)


def test_autotuner_picks_a_schedule(gpu_ctx, uneven_graphs):
    S, d, used, ms = solve_with(gpu_ctx, uneven_graphs, -1)
    assert used in (0, 2, 4, 5)
    assert ms[0] > 0 and ms[2] > 0 and ms[4] > 0 and ms[5] > 0
    _, d0, _, _ = solve_with(gpu_ctx, uneven_graphs, 0)
    for g in range(len(d)):
        assert np.array_equal(d[g], d0[g])


def test_many_graphs_full_frame(gpu_ctx, uneven_graphs):
    """The multi-iteration frame (iter = 12 graphs into one splat) renders and
    is identical whichever Floyd-Warshall schedule runs."""
    sc = uneven_graphs
    out = []
    for schedule in (0, 1, 3):
        scenes.load_into(gpu_ctx, sc)
        gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
        gpu_ctx.set_fw_schedule(schedule)
        gpu_ctx.frame_device(sc.opts, sc.max_connect)
        out.append(gpu_ctx.films(sc.opts))
    for k in ["rgba", "direct", "scatter", "emission"]:
        assert np.array_equal(getattr(out[0], k), getattr(out[1], k))
        assert np.array_equal(getattr(out[0], k), getattr(out[2], k))
    assert np.isfinite(out[0].rgba).all()


def test_graph_replay_matches_direct_launches(gpu_ctx):
    sc = scenes.small(n_points=300, width=48, height=40, spp=2)
    scenes.load_into(gpu_ctx, sc)
    gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    gpu_ctx.set_graph_mode(False)
    gpu_ctx.frame_device(sc.opts, sc.max_connect)
    ref = gpu_ctx.films(sc.opts)
    gpu_ctx.set_graph_mode(True)
    for _ in range(3):  # run + capture, then two replays
        gpu_ctx.frame_device(sc.opts, sc.max_connect)
        got = gpu_ctx.films(sc.opts)
        for k in ["rgba", "direct", "scatter", "emission"]:
            assert np.array_equal(getattr(got, k), getattr(ref, k)), k
    assert gpu_ctx.lib.lg_frame_launches(gpu_ctx.h) > 10
    gpu_ctx.set_graph_mode(False)


def inner_loop_sums_f32() -> np.ndarray:
    """The inner-loop probe's per-thread results, restated in FP32 numpy: the
    update tiles' 8 x 8 register tile per thread (rows rbase + 8q + {0, 1},
    columns cbase + 16q + {0, 1}), 32 k-pairs over the probe's fixed operand
    patterns, acc = min(acc, a.x + b.x, a.y + b.y), then the 64 values summed
    row by row. Every operand and sum is a small exact FP32 value."""
    e = np.arange(32 * 128)
    A = np.stack([(e * 37) % 101, (e * 53) % 97 + 0.25], -1).astype(np.float32).reshape(32, 128, 2)
    B = np.stack([(e * 29) % 89 + 0.5, (e * 61) % 83], -1).astype(np.float32).reshape(32, 128, 2)
    out = np.empty(256, np.float32)
    for tid in range(256):
        warp, lane = tid >> 5, tid & 31
        rbase = (warp >> 1) * 32 + (lane >> 3) * 2
        cbase = (warp & 1) * 64 + (lane & 7) * 2
        rows = np.array([rbase + 8 * (r >> 1) + (r & 1) for r in range(8)])
        cols = np.array([cbase + 16 * (c >> 1) + (c & 1) for c in range(8)])
        a, b = A[:, rows, :], B[:, cols, :]                      # [kp][8][2]
        s = a[:, :, None, :] + b[:, None, :, :]                  # [kp][r][c][2], FP32
        acc = np.minimum(np.float32(1e30), s.min(axis=(0, 3)))   # the init rounds to 1e30f
        tot = np.float32(0.0)
        for v in acc.reshape(-1):
            tot = np.float32(tot + v)
        out[tid] = tot
    return out


def test_fw_inner_loop_ceiling(gpu_ctx):
    """The min-plus inner loop alone: its results equal an FP32 restatement of
    the same packed adds and 3-input mins bit for bit, and it runs near half
    of the FMA-counted FP32 peak (an add and a min per update, each an FP32
    lane cycle): between 20 and 70 TFLOP/s on a GB300 (152 SMs, ~1.9-2.07
    GHz)."""
    t, sums = gpu_ctx.fw_inner_loop_rate(want_sums=True)
    assert np.array_equal(sums, inner_loop_sums_f32())
    assert 20.0 < t < 70.0, t


def test_fw_full_size_properties(gpu_ctx):
    """The production solve size (one 4096-point graph, 64 rounds), where the
    FP32 oracle would take minutes: size-independent properties instead.
    The symmetric persistent solve (schedule 4, what the autotuner picks) and
    the per-round launches (schedule 0) give the same bits; the result is
    exactly symmetric with a zero diagonal; finite entries are exactly the
    pairs the graph connects; and sampled triples satisfy the triangle
    inequality d_ij <= d_ik + d_kj (within 1e-6 relative: the solve rounds
    each path sum in its own association order)."""
    sc = scenes.small(n_points=4096, width=32, height=32, res=128)
    sc.radius = [0.06]
    scenes.load_into(gpu_ctx, sc)
    gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    S = gpu_ctx.march_edges(want=True)[0]
    assert S.shape == (4096, 4096)
    out = {}
    for schedule in (0, 4):
        gpu_ctx.march_edges()  # the solve works in place: start each from the edges
        gpu_ctx.set_fw_schedule(schedule)
        out[schedule] = gpu_ctx.solve_paths(want=True)[0]
        assert gpu_ctx.fw_schedule()[0] == schedule
    gpu_ctx.set_fw_schedule(-1)
    d = out[4]
    assert np.array_equal(d, out[0])
    assert np.array_equal(d, d.T)
    assert np.all(np.diag(d) == 0)
    fin = np.isfinite(d)
    # connectivity: finite exactly within the edge graph's components
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import connected_components
    _, label = connected_components(csr_matrix(np.isfinite(S)), directed=False)
    assert np.array_equal(fin, label[:, None] == label[None, :])
    assert np.all(d[np.isfinite(S)] <= S[np.isfinite(S)])
    rng = np.random.default_rng(7)
    i, j, k = (rng.integers(0, 4096, 200000) for _ in range(3))
    lhs = d[i, j].astype(np.float64)
    rhs = d[i, k].astype(np.float64) + d[k, j].astype(np.float64)
    ok = ~np.isfinite(rhs) | (lhs <= rhs * (1 + 1e-6))
    assert ok.all()


def test_fw_ragged_batch_edge_cases(gpu_ctx):
    """A batch with an empty graph, single points, sizes off the 64 / 128
    block grid and one that spans several rounds: the symmetric persistent
    solve (4, and 5 with TMA staging), the general one (2) and the per-round
    launches (0) agree bit for bit, and match the FP32 oracle within 1e-6."""
    sc = scenes.small(n_points=16, width=32, height=32)
    sizes = [0, 1, 2, 65, 129, 300, 1]
    sc.points = [scenes.points(sc.density.values, sc.density.voxel_size, n, seed=200 + g) if n > 0
                 else np.zeros((0, 3), np.float32) for g, n in enumerate(sizes)]
    sc.radius = [0.2] * len(sizes)
    sc.opts.iter = len(sizes)
    res = {}
    for schedule in (0, 2, 4, 5):
        S, dist, used, _ = solve_with(gpu_ctx, sc, schedule)
        assert used == schedule
        res[schedule] = (S, dist)
    gpu_ctx.set_fw_schedule(-1)
    S0, d0 = res[0]
    for schedule in (2, 4, 5):
        for g in range(len(sizes)):
            assert np.array_equal(res[schedule][1][g], d0[g]), (schedule, g)
    for g, n in enumerate(sizes):
        assert d0[g].shape == (n, n)
        if n == 0:
            continue
        ref = po.fw_minplus_f32(S0[g])
        np.fill_diagonal(ref, 0.0)
        fin = np.isfinite(ref)
        assert np.array_equal(np.isfinite(d0[g]), fin), g
        assert np.allclose(d0[g][fin], ref[fin], rtol=1e-6, atol=0), g
