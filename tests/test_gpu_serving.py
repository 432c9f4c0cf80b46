"""Serving: resident volumes, HBM-budget admission, concurrent requests.
A request's image must be the same alone and in the mix."""
import numpy as np
import pytest

from lightgraph_gb300 import LightGraphError, _capi
from lightgraph_gb300 import serve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_stream():
    vs = serve.make_volumes(None, resolutions=(32, 64), pool=1500)
    return vs


def test_mixed_equals_alone(small_stream):
    """Every result, environment-lit requests included, is bit-identical alone
    (one slot, its own path solve) and in the mix (four slots whose path
    solves share Floyd-Warshall launches)."""
    vs = small_stream
    alone_srv = serve.Server(max_inflight=1, solo_paths=True)
    mix_srv = serve.Server(max_inflight=4)
    try:
        for srv in (alone_srv, mix_srv):
            vs.ids = [srv.add_volume(g) for g in vs.grids]
            stream = serve.request_stream(vs, 8, rate=0, seed=4, n_min=64, n_max=600, images=(32, 48, 64),
                                          env_fraction=0.5)
            assert any(req.env_map is not None for _, req in stream)
            stats, imgs = serve.run_stream(srv, stream, want_images=True, realtime=False)
            assert stats["requests"] == 8
            if srv is mix_srv:
                # every request's graph went through a shared launch, and at
                # least one launch held more than one request's graph
                assert stats["path_graphs"] == 8 and stats["path_launches"] < 8
            if srv is alone_srv:
                alone = imgs
            else:
                mixed = imgs
        for a, b in zip(alone, mixed):
            assert a.shape == b.shape
            assert np.array_equal(a, b)
            assert np.isfinite(a).all()
    finally:
        alone_srv.close()
        mix_srv.close()


def test_budget_admission_and_errors(small_stream):
    vs = small_stream
    srv = serve.Server(max_inflight=3, queue_capacity=4, hbm_budget_bytes=64 << 20)
    try:
        vs.ids = [srv.add_volume(g) for g in vs.grids]
        stream = serve.request_stream(vs, 4, rate=0, seed=9, n_min=64, n_max=200, images=(32,))
        # a 64 MB budget admits these small requests one or two at a time;
        # all complete
        stats, imgs = serve.run_stream(srv, stream, want_images=True, realtime=False)
        assert all(np.isfinite(i).all() for i in imgs)
        # unknown ticket
        with pytest.raises(LightGraphError):
            srv.wait(123456, 0)
        with pytest.raises(LightGraphError):
            srv.poll(123456)
        # poll does not consume the result: a finished request polls done
        # until it is waited for, and is unknown after
        tk = srv.submit(stream[0][1])
        for _ in range(20000):
            if srv.poll(tk):
                break
            __import__("time").sleep(0.001)
        assert srv.poll(tk)
        img, _, _ = srv.wait(tk, 0)
        assert np.array_equal(img, imgs[0])
        with pytest.raises(LightGraphError):
            srv.poll(tk)
        # a request larger than the whole budget is refused up front
        big = serve.request_stream(vs, 1, rate=0, seed=1, n_min=3000, n_max=3000, images=(1024,))[0][1]
        with pytest.raises(LightGraphError) as e:
            srv.submit(big)
        assert e.value.status == _capi.LG_ERR_NOMEM
    finally:
        srv.close()


def test_queue_capacity(small_stream):
    vs = small_stream
    srv = serve.Server(max_inflight=1, queue_capacity=2)
    try:
        vs.ids = [srv.add_volume(g) for g in vs.grids]
        stream = serve.request_stream(vs, 12, rate=0, seed=5, n_min=400, n_max=600, images=(64,))
        tickets, busy = [], 0
        for _, req in stream:
            try:
                tickets.append(srv.submit(req))
            except LightGraphError as e:
                assert e.status == _capi.LG_ERR_BUSY
                busy += 1
        for t in tickets:
            srv.wait(t, -1, False)
        assert busy > 0 and len(tickets) + busy == 12
    finally:
        srv.close()


def test_env_light_needs_its_map(small_stream):
    vs = small_stream
    srv = serve.Server(max_inflight=1)
    try:
        vs.ids = [srv.add_volume(g) for g in vs.grids]
        req = serve.request_stream(vs, 1, rate=0, seed=2, n_min=64, n_max=64, images=(32,), env_fraction=1.0)[0][1]
        req.env_map = None
        with pytest.raises(LightGraphError) as e:
            srv.submit(req)
        assert e.value.status == _capi.LG_ERR_INVALID
    finally:
        srv.close()
