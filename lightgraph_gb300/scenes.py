"""Seeded synthetic scenes standing in for the reference's VDB/EXR assets.

The reference's scenes (scenes/*.sh) read OpenVDB clouds and EXR maps that it
does not ship. Each workload here is generated from a seed with the same
shapes and sizes instead (lightgraph_scene.h):

  small       128^3 dense sphere x 4-octave fBm (seed 0), voxel 0.01, extinction
              10 per world unit (-scattering 0.09 -absorption 0.01 per voxel
              step, albedo 0.9), one directional light, 1024 interior points
              connected within 0.15, 256x256 at 1 spp, camera on +z.
  production  512^3 sparse cumulus (8^3 leaves, ~14% active, 6-octave fBm seed
              1), voxel 0.0025, extinction 20 per world unit with RGB
              scattering scale (1.0, 1.1, 1.25), temperature fBm seed 2 in
              [0, 1500] through a 4-key ramp, one directional and one point
              light, 4096 points, 1024x1024 at 4 spp.
  envmap      the small scene with a 512x256 sky map (gradient + Gaussian sun,
              sigma 2 deg at 30 deg elevation) as an importance-sampled light.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from .lightgraph import ColorRamp, Grid, Light, SceneSettings, Shader


@dataclass
class Scene:
    name: str
    density: Grid
    temperature: Grid | None
    shader: Shader
    lights: list
    env_map: np.ndarray | None
    opts: SceneSettings
    points: list
    radius: list           # connection radius per graph (world units)
    max_connect: int = 12
    point_voxel_size: float = 0.0
    info: dict = field(default_factory=dict)

    @property
    def radius_sq(self):
        return [np.float32(r) * np.float32(r) for r in self.radius]


def volume(kind: int, res: int, octaves: int, seed: int, scale: float = 1.0, mask=None) -> np.ndarray:
    lib = _capi.load_host()
    out = np.empty((res, res, res), np.float32)
    m = None if mask is None else np.ascontiguousarray(mask, np.float32)
    lib.lgs_volume(kind, res, octaves, seed, scale, _capi.ptr(m), _capi.ptr(out))
    return out


def points(density: np.ndarray, voxel_size: float, n: int, seed: int) -> np.ndarray:
    lib = _capi.load_host()
    res = density.shape[0]
    out = np.empty((n, 3), np.float32)
    got = lib.lgs_points(_capi.ptr(np.ascontiguousarray(density)), res, voxel_size, n, seed, 1e-3, n * 100000,
                         _capi.ptr(out))
    return out[:got]


def envmap(w: int = 512, h: int = 256, elev: float = 30.0, azim: float = 60.0, sigma: float = 2.0,
           intensity: float = 50.0) -> np.ndarray:
    lib = _capi.load_host()
    out = np.empty((h, w, 3), np.float32)
    lib.lgs_envmap(w, h, elev, azim, sigma, intensity, _capi.ptr(out))
    return out


def _grid(vals: np.ndarray, voxel: float) -> Grid:
    r = vals.shape[0]
    return Grid(vals, (-r // 2, -r // 2, -r // 2), voxel)


def small(n_points: int = 1024, width: int = 256, height: int = 256, spp: int = 1, res: int = 128,
          seed: int = 0, radius: float = 0.15) -> Scene:
    voxel = 1.28 / res
    dens = volume(_capi.LGS_VOLUME_SPHERE_FBM, res, 4, 0)
    sh = Shader()
    # extinction 10 per world unit at voxel 0.01 -> 0.1 per voxel step
    k = 10.0 * voxel
    sh.setScattering(0.9 * k)
    sh.setAbsorption(0.1 * k)
    sh.setVolumeColor(1.0)
    sh.setScatterScale(4.0 * 0.9 * k / 1.5)  # the default 4.0 relative to the default scattering 1.5
    opts = SceneSettings(width=width, height=height, samples=spp, camTranslate=(0.0, 0.0, 2.2), iter=1, seed=seed)
    lights = [Light.parse("dir:0:1,1,1:1.0:-35,25,0")]
    pts = [points(dens, voxel, n_points, seed=1000 + seed)]
    return Scene("small", _grid(dens, voxel), None, sh, lights, None, opts, pts, [radius],
                 info={"res": res, "voxel": voxel, "active_voxels": int((dens > 0).sum())})


def production(n_points: int = 4096, width: int = 1024, height: int = 1024, spp: int = 4, res: int = 512,
               seed: int = 0, radius: float = 0.075) -> Scene:
    voxel = 1.28 / res
    dens = volume(_capi.LGS_VOLUME_CUMULUS, res, 6, 1)
    temp = volume(_capi.LGS_VOLUME_TEMPERATURE, res, 6, 2, 1500.0, mask=dens)
    sh = Shader()
    k = 20.0 * voxel  # extinction 20 per world unit
    sh.setScattering((0.9 * k * 1.0, 0.9 * k * 1.1, 0.9 * k * 1.25))
    sh.setAbsorption(0.1 * k)
    sh.setVolumeColor(1.0)
    sh.setScatterScale(4.0 * 0.9 * k / 1.5)
    sh.setEmissionScale(0.5)
    sh.setEmissionColorRamp(ColorRamp.parse(
        "0.0,0.33,0.66,1.0/0,0,0:1.0,0.076,0.0:1.0,0.322,0.0:1.0,0.45,0.15/600/1500"))
    opts = SceneSettings(width=width, height=height, samples=spp, camTranslate=(0.0, 0.0, 2.2), iter=1, seed=seed)
    lights = [Light.parse("dir:0:1,0.89,0.79:1.2:-40,30,0"), Light.parse("point:0:0.4,0.6,1.0:30:0.6,0.5,0.9")]
    pts = [points(dens, voxel, n_points, seed=2000 + seed)]
    return Scene("production", _grid(dens, voxel), _grid(temp, voxel), sh, lights, None, opts, pts, [radius],
                 info={"res": res, "voxel": voxel, "active_voxels": int((dens > 0).sum())})


def reference_scale(iterations: int = 500, width: int = 960, height: int = 540, spp: int = 3, res: int = 512,
                    seed: int = 0) -> Scene:
    """The reference's own workload shape (its explosion scene script): 500
    LightGraph iterations whose points come from dart throwing (~750 each, one
    splat of ~375k points), a distant light plus a 3-sample environment light,
    3 spp at the reference's default 960x540, ptsPerKernel 2, shadow step 2,
    cutoff 0.0025, on the production cumulus. The points are produced on the
    GPU (lg_scatter_graphs), so `points` is empty."""
    voxel = 1.28 / res
    dens = volume(_capi.LGS_VOLUME_CUMULUS, res, 6, 1)
    temp = volume(_capi.LGS_VOLUME_TEMPERATURE, res, 6, 2, 1500.0, mask=dens)
    sh = Shader()
    k = 20.0 * voxel
    sh.setScattering((0.9 * k * 1.0, 0.9 * k * 1.25, 0.9 * k * 1.5))
    sh.setAbsorption(0.1 * k)
    sh.setVolumeColor(1.0)
    sh.setDensityScale(0.5)
    sh.setScatterScale(3.0 * 0.9 * k / 1.5)
    sh.setScatterDensityScale(1.0)
    sh.setScatterDensityMin(0.025)
    sh.setScatterDensityMaskPower(1.0)
    sh.setEmissionScale(3.0)
    sh.setEmissionColorRamp(ColorRamp.parse(
        "0.0,0.33,0.66,1.0/0,0,0:1.0,0.076,0.0:1.0,0.322,0.0:1.0,0.45,0.15/600/1500"))
    opts = SceneSettings(width=width, height=height, samples=spp, camTranslate=(0.0, 0.0, 2.2), iter=iterations,
                         seed=seed, cutoff=0.0025, step=(1.0, 2.0), ptsPerKernel=2)
    lights = [Light.parse("dir:45:1,0.89,0.79:0.7:-48.8,-311.86,0"), Light.parse("env:0:1,1,1:0.35:3:sky")]
    return Scene("reference_scale", _grid(dens, voxel), _grid(temp, voxel), sh, lights, envmap(), opts, [], [],
                 info={"res": res, "voxel": voxel, "active_voxels": int((dens > 0).sum()),
                       "iterations": iterations})


def batched_graphs(n_graphs: int = 64, n_min: int = 256, n_max: int = 4096, seed: int = 3, res: int = 256,
                   radius: float = 0.15) -> Scene:
    """Many LightGraphs of uneven size solved together: n_graphs point sets
    with N log-uniform in [n_min, n_max] (seeded), all in one 256^3 fBm
    cumulus (one density grid per context), connect radius 0.15."""
    voxel = 1.28 / res
    dens = volume(_capi.LGS_VOLUME_CUMULUS, res, 6, 1)
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_graphs)).astype(int)
    pts = [points(dens, voxel, int(n), seed=3000 + seed * 1000 + g) for g, n in enumerate(sizes)]
    sh = Shader()
    k = 20.0 * voxel
    sh.setScattering((0.9 * k, 0.9 * k * 1.1, 0.9 * k * 1.25))
    sh.setAbsorption(0.1 * k)
    opts = SceneSettings(width=256, height=256, samples=1, camTranslate=(0.0, 0.0, 2.2), iter=n_graphs, seed=seed)
    lights = [Light.parse("dir:0:1,0.89,0.79:1.2:-40,30,0")]
    return Scene("batched_graphs", _grid(dens, voxel), None, sh, lights, None, opts, pts, [radius] * n_graphs,
                 info={"res": res, "voxel": voxel, "sizes": [int(len(p)) for p in pts]})


def with_envmap(scene: Scene, samples: int = 3) -> Scene:
    env = envmap()
    scene.lights = list(scene.lights) + [Light.parse(f"env:0:1,1,1:0.35:{samples}:sky")]
    scene.env_map = env
    return scene


def load_into(ctx, scene: Scene, dtype: int = _capi.LG_DTYPE_F32) -> None:
    """Uploads the scene's grids and settings into a Context."""
    ctx.upload_density(scene.density, dtype)
    ctx.upload_temperature(scene.temperature, dtype)
    ctx.set_shader(scene.shader)
    ctx.set_settings(scene.opts)
    ctx.set_lights(scene.lights, scene.env_map)
