"""Serving driver over the C ABI's lg_server_*: resident volumes, a Poisson
request stream, and latency / throughput statistics.

The workload stands in for a render service: four resident cumulus volumes
(64^3, 128^3, 256^3, 512^3), requests drawn uniformly over them with a
LightGraph of log-uniform [512, 8192] points, an image from {128^2, 256^2,
512^2, 1024^2} at 1-4 spp and 1-3 lights (a quarter of the requests add a
2-sample environment light on the synthetic 512x256 sky map), arriving as a
Poisson process.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import _capi, scenes
from ._capi import GridDesc, LightC, LightGraphError, RequestC, ServerOptsC, ptr
from .lightgraph import Grid, Light, SceneSettings, Shader


class Server:
    def __init__(self, device: int = 0, max_inflight: int = 4, queue_capacity: int = 1024,
                 hbm_budget_bytes: int = 64 << 30, solo_paths: bool = False):
        self.lib = _capi.load()
        o = ServerOptsC(device, max_inflight, queue_capacity, 1 if solo_paths else 0, hbm_budget_bytes)
        h = C.c_void_p()
        st = self.lib.lg_server_create(C.byref(o), C.byref(h))
        if st != _capi.LG_OK:
            raise LightGraphError(st, "lg_server_create failed")
        self.h = h
        self._keep = {}

    def _err(self, st):
        if st != _capi.LG_OK:
            raise LightGraphError(st, self.lib.lg_server_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.lg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_volume(self, density: Grid, temperature: Grid | None = None, dtype: int = _capi.LG_DTYPE_F32) -> int:
        d = density.desc()
        dv = np.ascontiguousarray(density.values, np.float32)
        t = temperature.desc() if temperature is not None else None
        tv = np.ascontiguousarray(temperature.values, np.float32) if temperature is not None else None
        vid = C.c_int32()
        self._err(self.lib.lg_server_add_volume(self.h, C.byref(d), ptr(dv), C.byref(t) if t is not None else None,
                                                ptr(tv), dtype, C.byref(vid)))
        return vid.value

    def submit(self, req: "Request") -> int:
        c = req.to_c()
        tk = C.c_int64()
        st = self.lib.lg_server_submit(self.h, C.byref(c), C.byref(tk))
        if st != _capi.LG_OK:
            self._err(st)
        self._keep[tk.value] = req
        return tk.value

    def stats(self):
        """(Floyd-Warshall launches, graphs they solved) so far."""
        a, b = C.c_uint64(), C.c_uint64()
        self._err(self.lib.lg_server_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def poll(self, ticket: int) -> bool:
        """True once the request has finished (its result stays for wait)."""
        done = C.c_int()
        st = self.lib.lg_server_poll(self.h, ticket, C.byref(done))
        if st != _capi.LG_OK:
            self._err(st)
        return bool(done.value)

    def wait(self, ticket: int, timeout_ms: int = -1, want_image: bool = True):
        req = self._keep.pop(ticket, None)
        img = None
        if want_image and req is not None:
            img = np.empty((req.opts.height, req.opts.width, 4), np.float32)
        q, lat = C.c_double(), C.c_double()
        st = self.lib.lg_server_wait(self.h, ticket, timeout_ms, ptr(img), C.byref(q), C.byref(lat))
        if st != _capi.LG_OK:
            if req is not None and st == _capi.LG_ERR_TIMEOUT:
                self._keep[ticket] = req
            self._err(st)
        return img, q.value, lat.value


@dataclass
class Request:
    volume: int
    points: list
    radius: list
    lights: list
    shader: Shader
    opts: SceneSettings
    max_connect: int = 12
    point_voxel_size: float = 0.0
    env_map: np.ndarray | None = None

    def to_c(self) -> RequestC:
        arrs = [np.ascontiguousarray(p, np.float32).reshape(-1, 3) for p in self.points]
        self._pts = np.ascontiguousarray(np.concatenate(arrs))
        self._offs = np.zeros(len(arrs) + 1, np.int64)
        self._offs[1:] = np.cumsum([len(a) for a in arrs])
        self._r2 = np.array([np.float32(r) * np.float32(r) for r in self.radius], np.float32)
        self._lights = (LightC * max(1, len(self.lights)))(*[l.c for l in self.lights])
        c = RequestC()
        c.volume = self.volume
        c.n_graphs = len(arrs)
        c.points = ptr(self._pts)
        c.offsets = ptr(self._offs)
        c.radius_sq = ptr(self._r2)
        c.max_connect = self.max_connect
        c.n_lights = len(self.lights)
        c.lights = C.cast(self._lights, C.c_void_p)
        c.shader = self.shader.to_c()
        c.settings = self.opts.to_c()
        c.camera = self.opts.camera_c()
        c.point_voxel_size = self.point_voxel_size
        if self.env_map is not None:
            self._env = np.ascontiguousarray(self.env_map, np.float32)
            c.env_rgb = ptr(self._env)
            c.env_h, c.env_w = self._env.shape[0], self._env.shape[1]
        return c


# ---------------------------------------------------------------------------
# the mixed workload
# ---------------------------------------------------------------------------

VOLUME_RES = (64, 128, 256, 512)
IMAGES = (128, 256, 512, 1024)
LIGHT_SPECS = ("dir:0:1,0.89,0.79:1.2:-40,30,0", "point:0:0.4,0.6,1.0:30:0.6,0.5,0.9",
               "dir:0:0.3,0.4,0.5:0.5:20,-120,0")
ENV_SPEC = "env:0:1,1,1:0.35:2:sky"
_SKY = None


def sky_map() -> np.ndarray:
    """The synthetic 512x256 sky map the environment-lit requests share."""
    global _SKY
    if _SKY is None:
        _SKY = scenes.envmap()
    return _SKY


@dataclass
class VolumeSet:
    ids: list
    grids: list
    pools: list  # interior points per volume (seeded)
    shaders: list


def make_volumes(server: Server | None, resolutions=VOLUME_RES, pool: int = 8192) -> VolumeSet:
    ids, grids, pools, shaders = [], [], [], []
    for k, res in enumerate(resolutions):
        voxel = 1.28 / res
        dens = scenes.volume(_capi.LGS_VOLUME_CUMULUS, res, 6, 10 + k)
        g = Grid(dens, (-res // 2,) * 3, voxel)
        if server is not None:
            ids.append(server.add_volume(g))
        grids.append(g)
        pools.append(scenes.points(dens, voxel, pool, seed=500 + k))
        sh = Shader()
        kk = 20.0 * voxel
        sh.setScattering((0.9 * kk, 0.99 * kk, 1.125 * kk))
        sh.setAbsorption(0.1 * kk)
        sh.setScatterScale(4.0 * 0.9 * kk / 1.5)
        shaders.append(sh)
    return VolumeSet(ids, grids, pools, shaders)


def request_stream(vs: VolumeSet, n: int, rate: float, seed: int = 4, n_min: int = 512, n_max: int = 8192,
                   images=IMAGES, env_fraction: float = 0.25):
    """(arrival time s, Request) pairs: Poisson arrivals at `rate` req/s. The
    requests themselves depend only on the seed, not on the rate."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n):
        gap = rng.exponential(1.0)  # drawn for every rate, so the requests do not depend on it
        t += gap / rate if rate > 0 else 0.0
        v = int(rng.integers(len(vs.grids)))
        npts = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        pool = vs.pools[v]
        npts = min(npts, len(pool))
        start = int(rng.integers(0, len(pool) - npts + 1))
        pts = pool[start:start + npts]
        img = int(images[int(rng.integers(len(images)))])
        spp = int(rng.integers(1, 5))
        nl = int(rng.integers(1, 4))
        lights = [Light.parse(s) for s in LIGHT_SPECS[:nl]]
        env = None
        if env_fraction > 0 and rng.random() < env_fraction:
            lights.append(Light.parse(ENV_SPEC))
            env = sky_map()
        # connection radius: 1.7 x the mean point spacing of the request
        spacing = (0.3 / max(npts, 1)) ** (1.0 / 3.0)
        opts = SceneSettings(width=img, height=img, samples=spp, camTranslate=(0.0, 0.0, 2.2), iter=1,
                             seed=1000 + q)
        out.append((t, Request(vs.ids[v] if vs.ids else v, [pts], [1.7 * spacing], lights, vs.shaders[v], opts,
                               env_map=env)))
    return out


def run_stream(server: Server, stream, want_images: bool = False, realtime: bool = True):
    """Submits at the arrival times (or all at once) and waits for all.
    Returns (stats, images)."""
    t0 = time.perf_counter()
    tickets = []
    for t_arr, req in stream:
        if realtime:
            dt = t_arr - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
        tickets.append(server.submit(req))
    lat, que, imgs = [], [], []
    for tk in tickets:
        img, q, l = server.wait(tk, -1, want_images)
        lat.append(l / 1e3)
        que.append(q / 1e3)
        imgs.append(img)
    wall = time.perf_counter() - t0
    lat = np.array(lat)
    stats = {"requests": len(stream), "wall_s": wall, "renders_per_s": len(stream) / wall,
             "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
             "mean_ms": float(lat.mean()), "queue_p50_ms": float(np.percentile(que, 50))}
    launches, graphs = server.stats()
    stats["path_launches"] = launches
    stats["path_graphs"] = graphs
    return stats, imgs


def run_standalone(vs: VolumeSet, stream, device: int = 0, fw_schedule: int = 4):
    """The plain drop-in path, one request at a time, as the reference runs one
    render per invocation: load the request's volume, then lg_render_frame with
    the request's points and lights (host buffers in, the four films out). One
    context is reused (no CUDA context per request) and the Floyd-Warshall
    schedule is fixed to the server's (no autotuning per size). The volume
    load (lg_upload_grid and the scene settings) is timed apart from the
    render. All requests are taken at once (throughput when the queue never
    drains)."""
    from .lightgraph import Context
    ctx = Context(device)
    ctx.set_fw_schedule(fw_schedule)
    t0 = time.perf_counter()
    lat, up = [], []
    for _, req in stream:
        t = time.perf_counter()
        ctx.upload_density(vs.grids[vs.ids.index(req.volume) if vs.ids else req.volume])
        ctx.set_shader(req.shader)
        ctx.set_settings(req.opts)
        ctx.set_lights(req.lights, req.env_map)
        t1 = time.perf_counter()
        r2 = [np.float32(r) * np.float32(r) for r in req.radius]
        ctx.render_frame(req.points, r2, req.opts, req.max_connect, req.point_voxel_size)
        t2 = time.perf_counter()
        up.append((t1 - t) * 1e3)
        lat.append((t2 - t1) * 1e3)
    wall = time.perf_counter() - t0
    ctx.close()
    lat, up = np.array(lat), np.array(up)
    render_s = float(lat.sum()) / 1e3
    return {"requests": len(stream), "wall_s": wall, "renders_per_s": len(stream) / wall,
            "renders_per_s_without_upload": len(stream) / render_s, "upload_ms_mean": float(up.mean()),
            "fw_schedule": fw_schedule, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean())}
