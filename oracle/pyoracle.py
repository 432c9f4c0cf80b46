"""ctypes binding of the CPU oracle (oracle/lg_oracle.h).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the reference results the GPU path is
compared with, or as the timed CPU baseline. The product package
(lightgraph_gb300) never imports it.

PARITY UNPINNED: the reference has no tests or fixtures and cannot be built
here, except its RandGen, against which the random sequence is pinned; see
lg_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from lightgraph_gb300 import build as _build  # noqa: E402  (build recipe only)
from lightgraph_gb300._capi import CameraC, GridDesc, LightC, SettingsC, ShaderC  # noqa: E402  (struct layouts)


class OGrid(C.Structure):
    _fields_ = [("desc", GridDesc), ("values", C.c_void_p)]


class OEnv(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("w", C.c_int32), ("h", C.c_int32)]


P = C.c_void_p
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.oracle_path()
    if not os.path.exists(path):
        _build.build_oracle()
    lib = C.CDLL(path)
    lib.lgo_build_graph.restype = C.c_int64
    lib.lgo_build_graph.argtypes = [C.c_int, P, C.c_float, C.c_int, P]
    lib.lgo_march_edges.restype = None
    lib.lgo_march_edges.argtypes = [C.POINTER(OGrid), C.POINTER(ShaderC), C.POINTER(SettingsC), C.c_int, P, P, P, P]
    lib.lgo_fw_maxtimes.argtypes = [C.c_int, P]
    lib.lgo_fw_minplus_f32.argtypes = [C.c_int, P]
    lib.lgo_fw_minplus_f64.argtypes = [C.c_int, P]
    lib.lgo_vertex_light.argtypes = [C.POINTER(OGrid), C.POINTER(OGrid), C.POINTER(ShaderC), C.POINTER(SettingsC),
                                     C.POINTER(LightC), C.c_int, C.POINTER(OEnv), C.c_int, P, C.c_int, P]
    lib.lgo_diffuse.argtypes = [C.c_int, P, P, P]
    lib.lgo_point_voxel_size.restype = C.c_double
    lib.lgo_point_voxel_size.argtypes = [C.c_int64, P, C.c_int]
    lib.lgo_splat.restype = C.c_double
    lib.lgo_splat.argtypes = [C.POINTER(OGrid), C.c_int, C.c_int64, P, P, C.c_double, C.c_double, P, P, P]
    lib.lgo_render.argtypes = [C.POINTER(OGrid), C.POINTER(OGrid), C.POINTER(ShaderC), C.POINTER(SettingsC),
                               C.POINTER(LightC), C.c_int, C.POINTER(OEnv), C.POINTER(CameraC), P, P, C.c_double, P,
                               C.c_int, C.c_int, P, P, P, P, P]
    lib.lgo_render_rows.argtypes = [C.POINTER(OGrid), C.POINTER(OGrid), C.POINTER(ShaderC), C.POINTER(SettingsC),
                                    C.POINTER(LightC), C.c_int, C.POINTER(OEnv), C.POINTER(CameraC), P, P,
                                    C.c_double, P, P, C.c_int, P, P, P, P, P]
    lib.lgo_env_cdf.argtypes = [C.POINTER(OEnv), P, P, P, P, P, P]
    lib.lgo_threads.restype = C.c_int
    lib.lgo_scatter_points.argtypes = [C.POINTER(OGrid), C.c_void_p, C.c_int, C.c_int, P, P, P]
    lib.lgo_randgen_draws.argtypes = [C.c_uint32, C.c_int64, P, P]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


class Oracle:
    """Holds one scene (grids, shader, settings, lights) and runs the
    reference's stages on the CPU in FP64."""

    def __init__(self, density, shader, opts, lights=(), temperature=None, env_map=None):
        self.lib = load()
        self._keep = []
        self.dens = self._grid(density)
        self.temp = self._grid(temperature) if temperature is not None else None
        self.shader = shader.to_c()
        self.settings = opts.to_c()
        self.opts = opts
        self.lights = (LightC * max(1, len(lights)))(*[l.c for l in lights])
        self.n_lights = len(lights)
        if env_map is not None:
            env = np.ascontiguousarray(env_map, np.float32)
            self._keep.append(env)
            self.env = OEnv(env.ctypes.data, env.shape[1], env.shape[0])
        else:
            self.env = None

    def _grid(self, g):
        vals = np.ascontiguousarray(g.values, np.float32)
        self._keep.append(vals)
        if g.leaf_mask is not None:
            self._keep.append(g.leaf_mask)
        return OGrid(g.desc(), vals.ctypes.data)

    def threads(self) -> int:
        return self.lib.lgo_threads()

    def build_graph(self, pts, radius_sq, max_connect=12):
        pts = np.ascontiguousarray(pts, np.float32)
        n = len(pts)
        adj = np.zeros((n, n), np.uint8)
        ne = self.lib.lgo_build_graph(n, _p(pts), C.c_float(radius_sq), max_connect, _p(adj))
        return adj, ne

    def march_edges(self, pts, adj, want_T=True):
        pts = np.ascontiguousarray(pts, np.float32)
        n = len(pts)
        T = np.zeros((n, n, 3)) if want_T else None
        S = np.zeros((n, n))
        self.lib.lgo_march_edges(C.byref(self.dens), C.byref(self.shader), C.byref(self.settings), n, _p(pts),
                                 _p(np.ascontiguousarray(adj, np.uint8)), _p(T), _p(S))
        return T, S

    def fw_maxtimes(self, T):
        T = np.ascontiguousarray(T, np.float64).copy()
        self.lib.lgo_fw_maxtimes(T.shape[0], _p(T))
        return T

    def vertex_light(self, pts, graph_id=0):
        pts = np.ascontiguousarray(pts, np.float32)
        L = np.zeros((len(pts), 3))
        self.lib.lgo_vertex_light(C.byref(self.dens), C.byref(self.temp) if self.temp else None,
                                  C.byref(self.shader), C.byref(self.settings), self.lights, self.n_lights,
                                  C.byref(self.env) if self.env else None, len(pts), _p(pts), graph_id, _p(L))
        return L

    def diffuse(self, T_solved, L):
        n = T_solved.shape[0]
        D = np.zeros((n, 3))
        self.lib.lgo_diffuse(n, _p(np.ascontiguousarray(T_solved, np.float64)),
                             _p(np.ascontiguousarray(L, np.float64)), _p(D))
        return D

    def splat(self, pts, D, point_voxel_size=None, factor=None, kernel_points=None):
        """ScatterGrid topology and splat of the points' radiance D. The point
        index's voxel size is the oracle's own computeVoxelSize of the points
        unless given."""
        pts = np.ascontiguousarray(pts, np.float32)
        if point_voxel_size is None:
            point_voxel_size = point_voxel_size_of(pts)
        D = np.ascontiguousarray(D, np.float64)
        f = factor or self.opts.scatterGridResFactor
        K = kernel_points if kernel_points is not None else self.opts.ptsPerKernel * self.opts.iter
        lo = (C.c_int32 * 3)()
        dims = (C.c_int32 * 3)()
        d = self.dens.desc
        box = []
        for a in range(3):
            l = (d.origin[a] // f) - 1
            h = (d.origin[a] + d.dims[a] - 1) // f + 1
            box.append(h - l + 1)
        out = np.zeros((box[2], box[1], box[0], 3))
        r = self.lib.lgo_splat(C.byref(self.dens), f, len(pts), _p(pts), _p(D), point_voxel_size, K, lo, dims,
                               _p(out))
        return tuple(lo), tuple(dims), out, r

    def render(self, sg=None, rows=None, counters=False):
        """sg = (lo, dims, values (z,y,x,3)) of the scatter grid, or None.
        rows: None (the whole image), a (first, end) pair, or a list of row
        indices (only those rows of the films are written)."""
        cam = self.opts.camera_c()
        W, H = self.opts.width, self.opts.height
        row_list = None
        if rows is not None and not (isinstance(rows, tuple) and len(rows) == 2):
            row_list = np.ascontiguousarray(rows, np.int32)
            r0 = r1 = 0
        else:
            r0, r1 = (0, H) if rows is None else rows
        films = [np.zeros((H, W, 4), np.float32) for _ in range(4)]
        cnt = np.zeros(2, np.uint64)
        if sg is not None:
            lo, dims, vals = sg
            vals32 = np.ascontiguousarray(vals, np.float32)
            lo_c, dims_c = (C.c_int32 * 3)(*lo), (C.c_int32 * 3)(*dims)
            sg_h = self.dens.desc.voxel_size * self.opts.scatterGridResFactor
        else:
            vals32, lo_c, dims_c, sg_h = None, None, None, 1.0
        args = (C.byref(self.dens), C.byref(self.temp) if self.temp else None, C.byref(self.shader),
                C.byref(self.settings), self.lights, self.n_lights, C.byref(self.env) if self.env else None,
                C.byref(cam), lo_c, dims_c, sg_h, _p(vals32))
        if row_list is None:
            self.lib.lgo_render(*args, r0, r1, *[_p(f) for f in films], _p(cnt))
        else:
            self.lib.lgo_render_rows(*args, _p(row_list), len(row_list), *[_p(f) for f in films], _p(cnt))
        return (films, cnt) if counters else films

    def env_cdf(self):
        w, h = self.env.w, self.env.h
        cf = np.zeros((h, w), np.float32)
        cc = np.zeros((h, w + 1), np.float32)
        ci = np.zeros(h, np.float32)
        mf = np.zeros(h, np.float32)
        mc = np.zeros(h + 1, np.float32)
        mi = np.zeros(1, np.float32)
        self.lib.lgo_env_cdf(C.byref(self.env), *[_p(x) for x in (cf, cc, ci, mf, mc, mi)])
        return cf, cc, ci, mf, mc, mi[0]


def scatter_points(density, opts, first_iter, n_iter):
    """lgo_scatter_points: (points n_iter x hard_limit x 3, counts, last squared minimum distance)."""
    lib = load()
    vals = np.ascontiguousarray(density.values, np.float32)
    g = OGrid(density.desc(), vals.ctypes.data)
    pts = np.zeros((n_iter, opts.hard_limit, 3), np.float32)
    cnt = np.zeros(n_iter, np.int32)
    m2 = np.zeros(n_iter, np.float32)
    lib.lgo_scatter_points(C.byref(g), C.cast(C.pointer(opts), C.c_void_p), first_iter, n_iter, _p(pts), _p(cnt),
                           _p(m2))
    return pts, cnt, m2


def randgen_draws(seed, n):
    """std::mt19937(seed) through std::uniform_real_distribution<float>(0, 1): (floats, raw)."""
    out = np.zeros(n, np.float32)
    raw = np.zeros(n, np.uint32)
    load().lgo_randgen_draws(seed, n, _p(out), _p(raw))
    return out, raw


def point_voxel_size_of(pts, points_per_voxel=8):
    """lgo_point_voxel_size: computeVoxelSize of an (n, 3) float32 point set."""
    pts = np.ascontiguousarray(pts, np.float32)
    return load().lgo_point_voxel_size(len(pts), _p(pts), points_per_voxel)


def diffuse(T_solved, L):
    """lgo_diffuse: diffuseLight on an RGB path matrix (diagonal 1) and vertex radiance."""
    n = T_solved.shape[0]
    D = np.zeros((n, 3))
    load().lgo_diffuse(n, _p(np.ascontiguousarray(T_solved, np.float64)), _p(np.ascontiguousarray(L, np.float64)),
                       _p(D))
    return D


def apsp_dijkstra_f64(S, sources=None):
    """Exact FP64 shortest path lengths of an optical-depth matrix S (+inf =
    no edge) by Dijkstra (scipy), from every vertex or from `sources`;
    diagonal 0. The min-plus form of floydAlgo's solution at sizes where the
    O(n^3) loops are too slow for a test (max-times FW = min-plus on
    -ln T, checked in tests/test_oracle.py)."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import dijkstra
    S = np.asarray(S, np.float64)
    fin = np.isfinite(S)
    np.fill_diagonal(fin, False)
    i, j = np.nonzero(fin)
    # explicit zeros are edges for scipy only when stored; keep every edge > 0
    w = np.maximum(S[i, j], np.finfo(np.float64).tiny)
    g = csr_matrix((w, (i, j)), shape=S.shape)
    return dijkstra(g, directed=True, indices=sources)


def transmittance_of(dist, extinction):
    """RGB path transmittance exp(extinction_c * dist) with diagonal 1 (the
    matrix floydAlgo leaves for diffuseLight)."""
    n = dist.shape[0]
    a = np.asarray(extinction, np.float64)
    T = np.exp(a[None, None, :] * np.asarray(dist, np.float64)[:, :, None])
    idx = np.arange(n)
    T[idx, idx, :] = 1.0
    return T


def fw_minplus_f32(S):
    S = np.ascontiguousarray(S, np.float32).copy()
    load().lgo_fw_minplus_f32(S.shape[0], _p(S))
    return S


def fw_minplus_f64(S):
    S = np.ascontiguousarray(S, np.float64).copy()
    load().lgo_fw_minplus_f64(S.shape[0], _p(S))
    return S


def build_graph(pts, radius_sq, max_connect=12):
    pts = np.ascontiguousarray(pts, np.float32)
    n = len(pts)
    adj = np.zeros((n, n), np.uint8)
    ne = load().lgo_build_graph(n, _p(pts), C.c_float(radius_sq), max_connect, _p(adj))
    return adj, ne
