"""Generates tests/golden/*.npz from the CPU oracle.

The reference ships no fixtures and cannot be built here, so these vectors are
the oracle's own outputs on small seeded scenes. They freeze the oracle (a
change to its arithmetic shows up as a mismatch) and give the GPU tests a
committed target. Regenerate with:

    python tests/golden/make_golden.py

Scenes:
  small_n96   : the small 128^3 sphere-fBm scene, 96 points, 24x24 at 2 spp
  env_n64     : the same volume with the sky map as an env light (2 samples),
                64 points, 16x16 at 1 spp
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lightgraph_gb300 import scenes  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def scene(name: str):
    if name == "small_n96":
        return scenes.small(n_points=96, width=24, height=24, spp=2, radius=0.3)
    if name == "env_n64":
        sc = scenes.small(n_points=64, width=16, height=16, spp=1, radius=0.3)
        return scenes.with_envmap(sc, samples=2)
    raise KeyError(name)


def compute(name: str) -> dict:
    sc = scene(name)
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights, temperature=sc.temperature, env_map=sc.env_map)
    pts = sc.points[0]
    adj, ne = o.build_graph(pts, sc.radius_sq[0], sc.max_connect)
    T, S = o.march_edges(pts, adj)
    Tsol = o.fw_maxtimes(T)
    Smin = po.fw_minplus_f64(S)
    L = o.vertex_light(pts)
    D = o.diffuse(Tsol, L)
    hp = po.point_voxel_size_of(pts)
    lo, dims, sg, radius = o.splat(pts, D, hp)
    films = o.render((lo, dims, sg))
    return {"points": pts, "radius_sq": np.float32(sc.radius_sq[0]), "adj": adj, "n_edges": np.int64(ne),
            "S": S, "T_solved": Tsol, "S_solved": Smin, "L": L, "D": D, "point_voxel_size": np.float64(hp),
            "sg_lo": np.array(lo), "sg_dims": np.array(dims), "scatter_grid": sg.astype(np.float32),
            "splat_radius": np.float64(radius), "rgba": films[0], "direct": films[1], "scatter": films[2],
            "emission": films[3]}


NAMES = ["small_n96", "env_n64"]


def main():
    for name in NAMES:
        data = compute(name)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
