"""The C-ABI library: loads without a GPU, exports every declared symbol, and
its host helpers mirror the reference's scene description."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from lightgraph_gb300 import _capi
from lightgraph_gb300.lightgraph import ColorRamp, Light, Shader

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("lightgraph_c.h", "lightgraph_scene.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b((?:lg|lgs)_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol():
    """Every function the headers declare is exported by the library whose
    ctypes table lists it: the CUDA library or the host-only helper library
    (which has no CUDA code, so a CPU-only caller can build scenes with it)."""
    lib, host = _capi.load(), _capi.load_host()
    names = declared_functions()
    assert len(names) > 30
    tables = set(_capi.SIGNATURES) | set(_capi.HOST_SIGNATURES)
    assert names <= tables, sorted(names - tables)
    assert not set(_capi.SIGNATURES) & set(_capi.HOST_SIGNATURES)
    missing = [n for n in sorted(names) if not hasattr(lib if n in _capi.SIGNATURES else host, n)]
    assert not missing, missing


def test_host_library_has_no_cuda_dependency():
    """The host helper library links no CUDA runtime, so the CPU baseline can
    build its scenes without mapping the CUDA library."""
    import subprocess
    from lightgraph_gb300 import build
    out = subprocess.run(["ldd", build.host_lib_path()], capture_output=True, text=True).stdout
    assert "cuda" not in out.lower() and "lightgraph_gb300" not in out


def test_version_and_no_device_is_reported():
    lib = _capi.load()
    assert b"sm_103a" in lib.lg_version()
    h = C.c_void_p()
    st = lib.lg_create(0, C.byref(h))
    if st == _capi.LG_OK:  # running on a GPU host
        lib.lg_destroy(h)
    else:
        assert st == _capi.LG_ERR_NODEVICE


def test_server_entry_points_reject_null_handles():
    """The serving calls check their handle and out-pointers before any
    device work (no GPU needed)."""
    lib = _capi.load()
    done = C.c_int(7)
    assert lib.lg_server_poll(None, 0, C.byref(done)) == _capi.LG_ERR_INVALID
    assert done.value == 7
    assert lib.lg_server_wait(None, 0, 0, None, None, None) == _capi.LG_ERR_INVALID
    tk = C.c_int64()
    assert lib.lg_server_submit(None, None, C.byref(tk)) == _capi.LG_ERR_INVALID
    assert lib.lg_server_destroy(None) in (_capi.LG_OK, _capi.LG_ERR_INVALID)


def request_bytes_restated(sizes, max_connect, width, height, spp, env_wh=None):
    """The serving admission estimate (lg_request_bytes) restated: per graph
    its padded FP32 matrix and edge slots; per point its position,
    candidates, graph id, vertex vectors and diffusion partial sums; per pixel
    the four films; per pixel sample its count, offset and primary results;
    the point bins; the env map with its CDFs."""
    b = 0
    for n in sizes:
        ld = (max(n, 1) + 127) // 128 * 128
        b += ld * ld * 4 + n * max_connect // 2 * 8
    P = sum(sizes)
    b += P * (12 + 96 * 2 + 4 + 4) + P * 4 * (3 + 3 + 3 + 3 * 16)
    b += width * height * 64 + width * height * max(spp, 1) * 44
    b += 160 * 160 * 160 * 12
    if env_wh:
        w, h = env_wh
        b += w * h * 4 * 5 + h * 4 * 262
    return b


def test_request_bytes_admission_estimate():
    """lg_request_bytes, the HBM estimate the server admits requests by, is
    pure host arithmetic (no GPU needed): it matches its restatement, grows
    with the graphs and the image, and is 0 for a request without graphs."""
    lib = _capi.load()

    def make(sizes, mc, w, h, spp, env=None):
        offs = np.zeros(len(sizes) + 1, np.int64)
        offs[1:] = np.cumsum(sizes)
        q = _capi.RequestC()
        q.n_graphs = len(sizes)
        q.offsets = offs.ctypes.data
        q.max_connect = mc
        q.camera.width, q.camera.height, q.camera.samples = w, h, spp
        if env is not None:
            q.env_rgb = env.ctypes.data
            q.env_h, q.env_w = env.shape[0], env.shape[1]
        return q, offs

    cases = [([100, 300], 12, 64, 32, 2, None), ([4096], 12, 1024, 1024, 4, None),
             ([0, 1, 129], 0, 16, 16, 0, None), ([512], 7, 128, 128, 1, (8, 4))]
    for sizes, mc, w, h, spp, env_wh in cases:
        env = np.zeros((env_wh[1], env_wh[0], 3), np.float32) if env_wh else None
        q, offs = make(sizes, mc, w, h, spp, env)
        assert lib.lg_request_bytes(C.byref(q)) == request_bytes_restated(sizes, mc, w, h, spp, env_wh)
    small, _o1 = make([256], 12, 64, 64, 1)
    big, _o2 = make([256, 2048], 12, 256, 256, 4)
    assert lib.lg_request_bytes(C.byref(big)) > lib.lg_request_bytes(C.byref(small))
    empty = _capi.RequestC()
    assert lib.lg_request_bytes(C.byref(empty)) == 0
    assert lib.lg_request_bytes(None) == 0


def test_noalloc_diffuse_argument_checks():
    """lg_diffuse_noalloc validates its arguments before touching the device:
    bad sizes, a leading dimension below n, null buffers and a positive
    extinction are refused, and n == 0 is a no-op (no GPU needed)."""
    lib = _capi.load()
    ext = (C.c_double * 3)(-1.0, -1.0, -1.0)
    buf = C.c_void_p(16)  # never dereferenced: every call below returns before any device work
    call = lib.lg_diffuse_noalloc
    assert call(None, 0, 0, None, None, ext, None) == _capi.LG_OK
    assert call(buf, -1, 0, buf, buf, ext, None) == _capi.LG_ERR_INVALID
    assert call(buf, 8193, 8193, buf, buf, ext, None) == _capi.LG_ERR_INVALID
    assert call(buf, 10, 9, buf, buf, ext, None) == _capi.LG_ERR_INVALID
    assert call(None, 10, 10, buf, buf, ext, None) == _capi.LG_ERR_INVALID
    assert call(buf, 10, 10, None, buf, ext, None) == _capi.LG_ERR_INVALID
    assert call(buf, 10, 10, buf, None, ext, None) == _capi.LG_ERR_INVALID
    assert call(buf, 10, 10, buf, buf, None, None) == _capi.LG_ERR_INVALID
    for bad in ((0.5, -1.0, -1.0), (-1.0, float("nan"), -1.0)):
        assert call(buf, 10, 10, buf, buf, (C.c_double * 3)(*bad), None) == _capi.LG_ERR_INVALID


def test_shader_defaults_and_coefficients():
    s = Shader()
    c = s.to_c()
    assert c.density_scale == 1.0 and c.density_max == 100.0 and c.scatter_density_scale == 0.35
    assert c.scatter_density_min == 0.025 and c.scatter_scale == 4.0 and c.scatter_density_mask_power == 0.25
    # albedo = color * s / (s + a), extinction = -(s + a)  (src/Shader.h:132-133)
    assert np.allclose(list(c.albedo), [1.5 / 1.6] * 3)
    assert np.allclose(list(c.extinction), [-1.6] * 3)
    s.setScattering((1.0, 1.25, 1.5))
    s.setAbsorption(0.5)
    s.setVolumeColor((0.5, 1.0, 2.0))
    c = s.to_c()
    assert np.allclose(list(c.albedo), [0.5 * 1 / 1.5, 1.25 / 1.75, 2 * 1.5 / 2.0])
    assert np.allclose(list(c.extinction), [-1.5, -1.75, -2.0])


def test_parse_lights():
    d = Light.parse("dir:0:1,0.5,0.25:0.7:0,0,0")
    assert d.type == _capi.LG_LIGHT_DISTANT
    assert np.allclose(list(d.c.dir), [0, 0, -1])
    assert np.allclose(list(d.c.color), [1, 0.5, 0.25])
    assert d.c.intensity == pytest.approx(np.float32(0.7))
    # directions stay unit length and the yRot turntable rotates about +y
    d2 = Light.parse("dir:90:1:1:0,0,0")
    assert np.allclose(np.linalg.norm(list(d2.c.dir)), 1.0)
    assert abs(d2.c.dir[1]) < 1e-12
    p = Light.parse("point:0:1,1,1:3:0.5,0.25,-1")
    assert p.type == _capi.LG_LIGHT_POINT and np.allclose(list(p.c.pos), [0.5, 0.25, -1])
    e = Light.parse("env:0:1,1,1:1.0:3:/some/map.exr")
    assert e.type == _capi.LG_LIGHT_ENV and e.c.samples == 3
    with pytest.raises(ValueError):
        Light.parse("spot:0:1:1:0,0,0")


def test_parse_color_ramp():
    r = ColorRamp.parse("0.0,0.33,0.66,1.0/0,0,0:1.0,0.076,0.0:1.0,0.322,0.0:1.0,0.45,0.15/0.35/1.5")
    assert r.positions == [0.0, 0.33, 0.66, 1.0]
    assert r.colors[1] == [1.0, 0.076, 0.0]
    assert (r.in_, r.out) == (0.35, 1.5)


def test_scene_generator_is_deterministic():
    from lightgraph_gb300 import scenes
    a = scenes.volume(_capi.LGS_VOLUME_SPHERE_FBM, 32, 4, 0)
    b = scenes.volume(_capi.LGS_VOLUME_SPHERE_FBM, 32, 4, 0)
    assert np.array_equal(a, b) and a.max() <= 1.0 and a.min() >= 0.0 and (a > 0).any()
    p = scenes.points(a, 0.04, 100, seed=5)
    q = scenes.points(a, 0.04, 100, seed=5)
    assert np.array_equal(p, q) and len(p) == 100


@pytest.mark.parametrize("sym", [0, 1])
@pytest.mark.parametrize("sizes", [[1], [64], [128], [200], [700], [4096], [0, 300, 33, 700, 129, 1000],
                                   [256, 4096, 512, 1300]])
def test_fw_queue_cannot_deadlock(sizes, sym):
    """The persistent solves' work queues, replayed on the host in order with
    the kernels' dependency waits: every wait is met by earlier items (so no
    residency can deadlock the launch) and every 64 x 64 block is written
    exactly once per round."""
    lib = _capi.load()
    arr = np.asarray(sizes, np.int32)
    n = C.c_int64()
    assert lib.lg_fw_queue_check(len(arr), arr.ctypes.data, sym, C.byref(n)) == _capi.LG_OK
    nts = [(s + 127) // 128 * 2 for s in sizes if s > 0]
    nus = [nt // 2 for nt in nts]
    if sym:
        # per round: nt - 1 column panel items (plus the diagonal item in
        # round 0; later diagonals close inside their strip item), nt - 1
        # strip blocks (all but the last round), the tiles on and above the
        # diagonal (rounds with nt >= 2)
        want = sum(1 + nt * (nt - 1) + (nt - 1) * (nt - 1) + (nt * nu * (nu + 1) // 2 if nt >= 2 else 0)
                   for nt, nu in zip(nts, nus))
    else:
        want = sum(nt * (2 * nt - 1) + (nt * nu * nu if nt >= 2 else 0) for nt, nu in zip(nts, nus))
    assert n.value == want


# the reference's command-line flags (src/main.cc:359-470)
REFERENCE_FLAGS = [
    "-absorption", "-camPos", "-camRot", "-camYRot", "-cutoff", "-densityMax", "-densityScale", "-emissionScale",
    "-exrOut", "-focal", "-geoDump", "-h", "-help", "-iter", "-light", "-primaryStep", "-ptsPerKernel", "-resHeight",
    "-resWidth", "-samples", "-scatterDensityMaskPower", "-scatterDensityMin", "-scatterDensityScale",
    "-scatterGridResFactor", "-scatterScale", "-scattering", "-shadowDensityScale", "-shadowStep",
    "-tempColorRamp", "-v", "-vdbIn", "-volumeColor",
]


def test_cli_help_lists_every_reference_flag():
    """The command-line renderer keeps the reference's flags (its scene
    scripts run unchanged apart from the input): its help, which needs no
    GPU, names every one of them (-vdbIn as unsupported without OpenVDB)."""
    import subprocess
    from lightgraph_gb300 import build
    build.build_library()
    r = subprocess.run([build.cli_path(), "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    words = set(re.findall(r"-[A-Za-z]+", r.stdout))
    missing = [f for f in REFERENCE_FLAGS if f not in words]
    assert not missing, missing
