"""Python mirror of the reference's hot-path interface over the C ABI.

The reference (asiroisvigneux/LightGraph) drives its multiple-scattering
estimate through three C++ classes: ``LightGraph`` (src/LightGraph.h:32-153),
``ScatterGrid`` (src/ScatterGrid.h:20-56) and ``VolumeRender``
(src/Renderer.h:403-448), configured by ``Shader`` (src/Shader.h:100-274),
``ColorRamp`` (src/Shader.h:23-93), the lights (src/Light.h) and
``SceneSettings`` (src/SceneSettings.h:21-63). This module keeps those names
and meanings; every computation runs in the CUDA library through
:class:`Context`. There is no CPU fallback: without the built library or a GPU
the calls raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _capi
from ._capi import CameraC, GridDesc, LightC, LightGraphError, SettingsC, ShaderC, ptr


def _check(lib, ctx, status: int) -> None:
    if status != _capi.LG_OK:
        msg = lib.lg_last_error(ctx).decode() if ctx else ""
        raise LightGraphError(status, msg)


# ---------------------------------------------------------------------------
# scene description
# ---------------------------------------------------------------------------

class ColorRamp:
    """ColorRamp(positions, colors, in, out) (src/Shader.h:41-48)."""

    def __init__(self, positions: Sequence[float] = (), colors: Sequence[Sequence[float]] = (),
                 in_: float = 0.0, out: float = 1.0):
        if len(positions) != len(colors):
            raise ValueError("positions and colors must have the same length")
        if len(positions) > _capi.LG_MAX_RAMP_KEYS:
            raise ValueError(f"at most {_capi.LG_MAX_RAMP_KEYS} ramp keys")
        self.positions = [float(p) for p in positions]
        self.colors = [[float(c) for c in col] for col in colors]
        self.in_ = float(in_)
        self.out = float(out)

    @classmethod
    def parse(cls, spec: str) -> "ColorRamp":
        """-tempColorRamp syntax (src/main.cc:280-319)."""
        lib = _capi.load_host()
        s = ShaderC()
        _check(lib, None, lib.lg_parse_color_ramp(spec.encode(), C.byref(s)))
        return cls([s.ramp_pos[k] for k in range(s.ramp_n)],
                   [[s.ramp_color[k][c] for c in range(3)] for k in range(s.ramp_n)], s.ramp_in, s.ramp_out)


class Shader:
    """The reference's built-in shader (src/Shader.h:100-274), same defaults,
    setters and derived albedo / extinction."""

    def __init__(self):
        self.density_scale = 1.0
        self.density_max = 100.0
        self.shadow_density_scale = 1.0
        self.scatter_density_scale = 0.35
        self.scatter_density_min = 0.025
        self.absorption = (0.1, 0.1, 0.1)
        self.scattering = (1.5, 1.5, 1.5)
        self.volume_color = (1.0, 1.0, 1.0)
        self.emission_scale = 0.0
        self.scatter_scale = 4.0
        self.scatter_density_mask_power = 0.25
        self.emission_color_ramp = ColorRamp()

    # setters named as in the reference
    def setDensityScale(self, v): self.density_scale = float(v)
    def setDensityMax(self, v): self.density_max = float(v)
    def setShadowDensityScale(self, v): self.shadow_density_scale = float(v)
    def setScatterDensityScale(self, v): self.scatter_density_scale = float(v)
    def setScatterDensityMin(self, v): self.scatter_density_min = float(v)
    def setAbsorption(self, v): self.absorption = _vec3(v)
    def setScattering(self, v): self.scattering = _vec3(v)
    def setVolumeColor(self, v): self.volume_color = _vec3(v)
    def setEmissionScale(self, v): self.emission_scale = float(v)
    def setEmissionColorRamp(self, r: ColorRamp): self.emission_color_ramp = r
    def setScatterScale(self, v): self.scatter_scale = float(v)
    def setScatterDensityMaskPower(self, v): self.scatter_density_mask_power = float(v)

    def getAlbedo(self):
        return tuple(c * s / (s + a) for c, s, a in zip(self.volume_color, self.scattering, self.absorption))

    def getExtinction(self):
        return tuple(-(s + a) for s, a in zip(self.scattering, self.absorption))

    def to_c(self) -> ShaderC:
        lib = _capi.load_host()
        s = ShaderC()
        lib.lg_shader_default(C.byref(s))
        s.density_scale = self.density_scale
        s.density_max = self.density_max
        s.shadow_density_scale = self.shadow_density_scale
        s.scatter_density_scale = self.scatter_density_scale
        s.scatter_density_min = self.scatter_density_min
        a, sc, col = ((C.c_double * 3)(*v) for v in (self.absorption, self.scattering, self.volume_color))
        lib.lg_shader_set_coefficients(C.byref(s), a, sc, col)
        s.emission_scale = self.emission_scale
        s.scatter_scale = self.scatter_scale
        s.scatter_density_mask_power = self.scatter_density_mask_power
        r = self.emission_color_ramp
        s.ramp_n = len(r.positions)
        for k, (p, col3) in enumerate(zip(r.positions, r.colors)):
            s.ramp_pos[k] = p
            for c in range(3):
                s.ramp_color[k][c] = col3[c]
        s.ramp_in = r.in_
        s.ramp_out = r.out
        return s


def _vec3(v):
    if np.isscalar(v):
        return (float(v),) * 3
    v = tuple(float(x) for x in v)
    if len(v) != 3:
        raise ValueError("expected 3 components")
    return v


class Light:
    """A light as parseLight builds it (src/main.cc:234-274), with the
    transform already applied. Use :meth:`parse` with the reference's -light
    syntax (plus ``point:yRot:r,g,b:intensity:x,y,z``)."""

    def __init__(self, c: LightC, spec: str = ""):
        self.c = c
        self.spec = spec

    @classmethod
    def parse(cls, spec: str) -> "Light":
        lib = _capi.load_host()
        c = LightC()
        st = lib.lg_parse_light(spec.encode(), C.byref(c))
        if st != _capi.LG_OK:
            raise ValueError(f"{spec} is not a valid light")
        return cls(c, spec)

    @property
    def type(self) -> int:
        return self.c.type


@dataclass
class SceneSettings:
    """SceneSettings (src/SceneSettings.h:21-63) plus the random-stream seed."""
    aperture: float = 36.0
    focal: float = 50.0
    znear: float = 1.0e-3
    zfar: float = float(np.finfo(np.float32).max)
    camRotate: tuple = (0.0, 0.0, 0.0)
    camTranslate: tuple = (0.0, 0.0, 0.0)
    camYRotate: float = 0.0
    samples: int = 1
    light: list = field(default_factory=list)
    cutoff: float = 0.005
    step: tuple = (1.0, 3.0)
    width: int = 960
    height: int = 540
    iter: int = 10
    scatterGridResFactor: int = 4
    ptsPerKernel: int = 3
    seed: int = 0

    def to_c(self) -> SettingsC:
        s = SettingsC()
        s.cutoff = self.cutoff
        s.step[0], s.step[1] = self.step
        s.iter = self.iter
        s.scatter_grid_res_factor = self.scatterGridResFactor
        s.pts_per_kernel = self.ptsPerKernel
        s.seed = self.seed
        return s

    def camera_c(self) -> CameraC:
        c = CameraC()
        for k in range(3):
            c.rotate[k] = self.camRotate[k]
            c.translate[k] = self.camTranslate[k]
        c.y_rotate = self.camYRotate
        c.focal = self.focal
        c.aperture = self.aperture
        c.znear = self.znear
        c.zfar = self.zfar
        c.width = self.width
        c.height = self.height
        c.samples = self.samples
        return c


@dataclass
class Grid:
    """A FloatGrid as a dense box: values[z, y, x] is the voxel at index
    origin + (x, y, z); world = index * voxel_size + world_origin."""
    values: np.ndarray
    origin: tuple
    voxel_size: float
    world_origin: tuple = (0.0, 0.0, 0.0)
    leaf_mask: np.ndarray | None = None

    def desc(self) -> GridDesc:
        d = GridDesc()
        nz, ny, nx = self.values.shape
        d.dims[0], d.dims[1], d.dims[2] = nx, ny, nz
        for a in range(3):
            d.origin[a] = int(self.origin[a])
            d.world_origin[a] = float(self.world_origin[a])
        d.voxel_size = float(self.voxel_size)
        d.leaf_mask = ptr(self.leaf_mask) if self.leaf_mask is not None else None
        return d


@dataclass
class Films:
    """The four Film objects of render() (src/main.cc:90-93), each H x W x 4."""
    rgba: np.ndarray
    direct: np.ndarray
    scatter: np.ndarray
    emission: np.ndarray


# ---------------------------------------------------------------------------
# device context
# ---------------------------------------------------------------------------

class Context:
    """One CUDA device and stream with the resident grids and stage buffers."""

    def __init__(self, device: int = 0):
        self.lib = _capi.load()
        h = C.c_void_p()
        st = self.lib.lg_create(device, C.byref(h))
        if st != _capi.LG_OK:
            raise LightGraphError(st, "lg_create failed (a CUDA device is required)")
        self.h = h
        self._graph_sizes: list[int] = []
        self._film_shape = (0, 0)

    def close(self) -> None:
        if self.h:
            self.lib.lg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, status: int) -> None:
        _check(self.lib, self.h, status)

    @property
    def stream(self) -> int:
        return self.lib.lg_stream(self.h)

    # scene
    def upload_grid(self, which: int, grid: Grid, dtype: int = _capi.LG_DTYPE_F32) -> None:
        vals = np.ascontiguousarray(grid.values, dtype=np.float32)
        d = grid.desc()
        self._ck(self.lib.lg_upload_grid(self.h, which, C.byref(d), ptr(vals), dtype))

    def upload_density(self, grid: Grid, dtype: int = _capi.LG_DTYPE_F32) -> None:
        self.upload_grid(_capi.LG_GRID_DENSITY, grid, dtype)

    def upload_temperature(self, grid: Grid | None, dtype: int = _capi.LG_DTYPE_F32) -> None:
        if grid is None:
            self._ck(self.lib.lg_clear_temperature(self.h))
        else:
            self.upload_grid(_capi.LG_GRID_TEMPERATURE, grid, dtype)

    def set_shader(self, shader: Shader) -> None:
        s = shader.to_c()
        self._ck(self.lib.lg_set_shader(self.h, C.byref(s)))

    def set_settings(self, opts: SceneSettings) -> None:
        s = opts.to_c()
        self._ck(self.lib.lg_set_settings(self.h, C.byref(s)))

    def set_lights(self, lights: Sequence[Light], env_map: np.ndarray | None = None) -> None:
        arr = (LightC * max(1, len(lights)))(*[l.c for l in lights])
        env = None if env_map is None else np.ascontiguousarray(env_map, dtype=np.float32)
        eh, ew = (0, 0) if env is None else env.shape[:2]
        self._ck(self.lib.lg_set_lights(self.h, arr, len(lights), ptr(env), ew, eh))

    # stage 1
    def scatter_points(self, first_iter: int, n_iter: int, opts: "_capi.ScatterOptsC | None" = None):
        """LightGraph::scatterPoints for iterations first_iter.. (see lg_scatter_points):
        returns (list of point arrays, radius_sq per iteration)."""
        o = opts if opts is not None else scatter_opts()
        pts = np.zeros((n_iter, o.hard_limit, 3), np.float32)
        cnt = np.zeros(n_iter, np.int32)
        r2 = np.zeros(n_iter, np.float32)
        self._ck(self.lib.lg_scatter_points(self.h, C.byref(o), first_iter, n_iter, _capi.ptr(pts), _capi.ptr(cnt),
                                            _capi.ptr(r2)))
        return [pts[i, :cnt[i]].copy() for i in range(n_iter)], r2

    def scatter_graphs(self, first_iter: int, n_iter: int, max_connect: int = 12,
                       opts: "_capi.ScatterOptsC | None" = None) -> np.ndarray:
        """scatter_points, then loads the iterations as graphs and connects
        them; returns the point count of each iteration."""
        o = opts if opts is not None else scatter_opts()
        cnt = np.zeros(n_iter, np.int32)
        self._ck(self.lib.lg_scatter_graphs(self.h, C.byref(o), first_iter, n_iter, max_connect, ptr(cnt)))
        self._graph_sizes = [int(c) for c in cnt]
        return cnt

    def build_graphs(self, points: Sequence[np.ndarray], radius_sq: Sequence[float], max_connect: int = 12,
                     want_adjacency: bool = False):
        pts, offs = _pack_points(points)
        r2 = np.asarray(radius_sq, dtype=np.float32)
        sizes = [len(p) for p in points]
        adj = np.zeros(sum(n * n for n in sizes), np.uint8) if want_adjacency else None
        ne = np.zeros(len(points), np.int64)
        self._ck(self.lib.lg_build_graphs(self.h, len(points), ptr(pts), ptr(offs), ptr(r2), max_connect,
                                          ptr(adj), ptr(ne)))
        self._graph_sizes = sizes
        out_adj = _split_square(adj, sizes) if adj is not None else None
        return out_adj, ne

    def _square_out(self, fn, want: bool):
        buf = np.empty(sum(n * n for n in self._graph_sizes), np.float32) if want else None
        self._ck(fn(self.h, ptr(buf)))
        return _split_square(buf, self._graph_sizes) if want else None

    def march_edges(self, want: bool = False):
        return self._square_out(self.lib.lg_march_edges, want)

    def solve_paths(self, want: bool = False):
        return self._square_out(self.lib.lg_solve_paths, want)

    def _vec_out(self, fn, want: bool):
        n = sum(self._graph_sizes)
        buf = np.empty((n, 3), np.float32) if want else None
        self._ck(fn(self.h, ptr(buf)))
        return buf

    def vertex_light(self, want: bool = False):
        return self._vec_out(self.lib.lg_vertex_light, want)

    def diffuse(self, want: bool = False):
        return self._vec_out(self.lib.lg_diffuse, want)

    def solve_graphs(self, want: bool = False):
        return self._vec_out(self.lib.lg_solve_graphs, want)

    def vertex_data(self):
        n = sum(self._graph_sizes)
        L = np.empty((n, 3), np.float32)
        D = np.empty((n, 3), np.float32)
        self._ck(self.lib.lg_get_vertex_data(self.h, ptr(L), ptr(D)))
        return L, D

    # stage 2
    def splat(self, point_voxel_size: float = 0.0) -> None:
        self._ck(self.lib.lg_splat(self.h, point_voxel_size))

    def scatter_grid(self):
        dims = (C.c_int32 * 3)()
        lo = (C.c_int32 * 3)()
        self._ck(self.lib.lg_get_scatter_grid(self.h, dims, lo, None))
        vals = np.empty((dims[2], dims[1], dims[0], 3), np.float32)
        self._ck(self.lib.lg_get_scatter_grid(self.h, dims, lo, ptr(vals)))
        return tuple(lo), tuple(dims), vals

    # stage 3
    def render(self, opts: SceneSettings) -> Films:
        cam = opts.camera_c()
        shape = (opts.height, opts.width, 4)
        films = [np.empty(shape, np.float32) for _ in range(4)]
        self._ck(self.lib.lg_render(self.h, C.byref(cam), *[ptr(f) for f in films]))
        return Films(*films)

    def render_wave_times(self):
        """Wave durations (ms) of the last render made with profiling on:
        primary count + scan, primary shading, shadow-ray ordering, shadow
        rays, resolve."""
        ms = (C.c_double * 5)()
        self._ck(self.lib.lg_render_wave_times(self.h, ms))
        return list(ms)

    def render_stats(self):
        """(primary density samples, shadow density samples) of the last render."""
        a, b = C.c_uint64(), C.c_uint64()
        self._ck(self.lib.lg_render_stats(self.h, C.byref(a), C.byref(b), None))
        return a.value, b.value

    def shading_tasks(self) -> int:
        """Primary samples of the last render that cast shadow rays."""
        t = C.c_uint64()
        self._ck(self.lib.lg_render_stats(self.h, None, None, C.byref(t)))
        return t.value

    def render_frame(self, points: Sequence[np.ndarray], radius_sq: Sequence[float], opts: SceneSettings,
                     max_connect: int = 12, point_voxel_size: float = 0.0) -> Films:
        pts, offs = _pack_points(points)
        r2 = np.asarray(radius_sq, dtype=np.float32)
        cam = opts.camera_c()
        shape = (opts.height, opts.width, 4)
        films = [np.empty(shape, np.float32) for _ in range(4)]
        self._ck(self.lib.lg_render_frame(self.h, len(points), ptr(pts), ptr(offs), ptr(r2), max_connect,
                                          point_voxel_size, C.byref(cam), *[ptr(f) for f in films]))
        self._graph_sizes = [len(p) for p in points]
        return Films(*films)

    def frame_device(self, opts: SceneSettings, max_connect: int = 12, point_voxel_size: float = 0.0) -> None:
        cam = opts.camera_c()
        self._ck(self.lib.lg_frame_device(self.h, max_connect, point_voxel_size, C.byref(cam)))

    def set_fw_schedule(self, schedule: int) -> None:
        """-1 autotuned, 0 per-graph launches, 1/2 persistent (CTAs per SM),
        3/4 symmetric persistent (CTAs per SM), 5 = 4 with the update tiles'
        operands staged by TMA bulk copies."""
        self._ck(self.lib.lg_set_fw_schedule(self.h, schedule))

    def fw_inner_loop_rate(self, want_sums: bool = False):
        """FP32 TFLOP/s (add + min per update) of the Floyd-Warshall update
        tiles' inner loop alone: the min-plus ceiling on this GPU. With
        want_sums, also each thread's sum of its final tile in the first CTA
        (256 floats), for checking the loop's arithmetic."""
        v = C.c_double()
        if not want_sums:
            self._ck(self.lib.lg_fw_inner_loop_rate(self.h, C.byref(v), None))
            return v.value
        sums = np.empty(256, np.float32)
        self._ck(self.lib.lg_fw_inner_loop_rate(self.h, C.byref(v), sums.ctypes.data))
        return v.value, sums

    def fw_schedule(self):
        s = C.c_int()
        ms = (C.c_double * 6)()
        self._ck(self.lib.lg_fw_schedule(self.h, C.byref(s), ms, 6))
        return s.value, list(ms)

    def set_graph_mode(self, on: bool) -> None:
        self._ck(self.lib.lg_set_graph_mode(self.h, 1 if on else 0))

    def films(self, opts: SceneSettings) -> Films:
        """The films of the last render or frame_device (waits for it)."""
        shape = (opts.height, opts.width, 4)
        films = [np.empty(shape, np.float32) for _ in range(4)]
        self._ck(self.lib.lg_get_films(self.h, *[ptr(f) for f in films]))
        return Films(*films)

    def fw_host(self, S: np.ndarray) -> np.ndarray:
        out = np.ascontiguousarray(S, dtype=np.float32).copy()
        self._ck(self.lib.lg_fw_host(self.h, ptr(out), out.shape[0]))
        return out

    def kernel_launches(self) -> int:
        return int(self.lib.lg_kernel_launches(self.h))


def _pack_points(points: Sequence[np.ndarray]):
    arrs = [np.ascontiguousarray(p, dtype=np.float32).reshape(-1, 3) for p in points]
    offs = np.zeros(len(arrs) + 1, np.int64)
    offs[1:] = np.cumsum([len(a) for a in arrs])
    pts = np.concatenate(arrs) if arrs else np.zeros((0, 3), np.float32)
    return np.ascontiguousarray(pts), offs


def _split_square(buf: np.ndarray, sizes: Sequence[int]):
    out, o = [], 0
    for n in sizes:
        out.append(buf[o:o + n * n].reshape(n, n))
        o += n * n
    return out


def scatter_opts(**kw) -> "_capi.ScatterOptsC":
    """The reference's dart-throwing constants (lg_scatter_opts_default), with overrides."""
    o = _capi.ScatterOptsC()
    _capi.load().lg_scatter_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def randgen_draws(seed: int, n: int):
    """RandGen::operator() for the engine seeded with seed: (floats, raw uint32)."""
    out = np.zeros(n, np.float32)
    raw = np.zeros(n, np.uint32)
    st = _capi.load().lg_randgen_draws(seed, n, _capi.ptr(out), _capi.ptr(raw))
    if st != 0:
        raise RuntimeError(f"lg_randgen_draws failed ({st})")
    return out, raw


# ---------------------------------------------------------------------------
# the reference's classes
# ---------------------------------------------------------------------------

class LightGraph:
    """LightGraph::operator() over all iterations (src/LightGraph.h:158-196):
    for each injected point cloud, buildGraph, raymarchConnection, floydAlgo,
    computeLighting and diffuseLight, all on the GPU. Returns the diffused
    vertex radiance per iteration (mDiffusePointGather)."""

    def __init__(self, ctx: Context, max_connect: int = 12):
        self.ctx = ctx
        self.max_connect = max_connect

    def scatterPoints(self, first_iter: int, n_iter: int = 1, opts=None):
        """LightGraph::scatterPoints (src/LightGraph.h:206-274) for n_iter
        iterations: the point clouds and each searchRadiusConnect."""
        pts, r2 = self.ctx.scatter_points(first_iter, n_iter, opts)
        return pts, [float(np.sqrt(np.float32(x))) for x in r2]

    def __call__(self, point_clouds: Sequence[np.ndarray], search_radius: Sequence[float]):
        r2 = [np.float32(r) * np.float32(r) for r in search_radius]
        self.ctx.build_graphs(point_clouds, r2, self.max_connect)
        D = self.ctx.solve_graphs(want=True)
        out, o = [], 0
        for p in point_clouds:
            out.append(D[o:o + len(p)])
            o += len(p)
        return out


class ScatterGrid:
    """ScatterGrid::buildScatterGrid + operator() (src/ScatterGrid.h:61-144):
    splats every solved vertex of the context into the coarse grid."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def __call__(self, point_voxel_size: float = 0.0):
        self.ctx.splat(point_voxel_size)
        return self.ctx.scatter_grid()


class VolumeRender:
    """VolumeRender::render (src/Renderer.h:496-693) on the context's grids."""

    def __init__(self, ctx: Context, opts: SceneSettings):
        self.ctx = ctx
        self.opts = opts

    def render(self) -> Films:
        return self.ctx.render(self.opts)
