"""The production frame at full size (512^3 sparse cumulus, one 4096-point
LightGraph, 1024x1024 at 4 spp, a distant and a point light), where the FP64
oracle would take minutes per frame: size-independent properties of the
render instead of a comparison with the oracle (the oracle comparisons run on
the small scenes of test_gpu_parity.py)."""
import numpy as np
import pytest

from lightgraph_gb300 import scenes

pytestmark = pytest.mark.gpu

FILMS = ["rgba", "direct", "scatter", "emission"]


@pytest.fixture(scope="module")
def production():
    return scenes.production()


def test_production_frame_properties(gpu_ctx, production):
    sc = production
    scenes.load_into(gpu_ctx, sc)
    gpu_ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    gpu_ctx.set_graph_mode(False)
    gpu_ctx.frame_device(sc.opts, sc.max_connect)
    a = gpu_ctx.films(sc.opts)
    prim, shad = gpu_ctx.render_stats()
    # deterministic: the same frame again, and replayed from a CUDA graph
    gpu_ctx.frame_device(sc.opts, sc.max_connect)
    b = gpu_ctx.films(sc.opts)
    gpu_ctx.set_graph_mode(True)
    for _ in range(2):  # run + capture, then a replay
        gpu_ctx.frame_device(sc.opts, sc.max_connect)
    c = gpu_ctx.films(sc.opts)
    gpu_ctx.set_graph_mode(False)
    for k in FILMS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
        assert np.array_equal(getattr(a, k), getattr(c, k)), k
        assert np.isfinite(getattr(a, k)).all(), k
    rgba = a.rgba
    assert rgba.shape == (1024, 1024, 4)
    alpha = rgba[..., 3]
    assert alpha.min() >= 0.0 and alpha.max() <= 1.0
    assert alpha.min() == 0.0          # background pixels see no cloud
    assert (alpha > 0.5).mean() > 0.05  # and the cloud covers part of the frame
    # rgb is the per-sample sum of the three AOVs (src/Renderer.h:674-677)
    total = a.direct[..., :3] + a.scatter[..., :3] + a.emission[..., :3]
    assert np.allclose(rgba[..., :3], total, rtol=1e-5, atol=1e-6)
    for k in FILMS:
        assert (getattr(a, k)[..., :3] >= 0).all(), k
    # the workload the bench quotes: ~98 M primary, ~3.4 G shadow samples
    assert 5e7 < prim < 2e8 and 1e9 < shad < 1e10
