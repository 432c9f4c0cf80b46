"""Benchmark of the LightGraph multiple-scattering frame on GB300.

Workload (one "step" = one frame): the 512^3 sparse cumulus (8^3 leaves, ~14%
active, 6-octave fBm seed 1, extinction 20 / world unit, RGB scattering scale
1.0/1.1/1.25) with a temperature grid through a 4-key ramp, one directional
and one point light, one LightGraph of 4096 points (a 64 MB FP32 distance
matrix), 1024x1024 at 4 spp, FP32 throughout. Inputs are seeded synthetic
stand-ins for the reference's VDB assets. The density grid in its brick layout
(~575 MB) is larger than L2, so no L2 flush is needed between steps.

  value : ms per frame with the grids and points resident in HBM (CUDA events on
          the library's stream around K frames); a frame is graph build, edge
          march, Floyd-Warshall, vertex light, diffusion, splat and render.
  e2e   : ms per frame through the public C ABI (lg_render_frame) with the points
          copied in from pinned host memory and the four films copied back.
  --impl reference : the reference's CPU path as restated by the oracle (FP64,
          OpenMP over all host cores), on a bounded sample scaled to ms/frame
          (the sampling rule is checked against one whole frame in the same
          run); the default run's cpu_baseline times one whole frame.

Multi-GPU: graphs and frames are independent, so N ranks run N replicas (one
frame each per step, no collective); value = wall ms per frame of the job.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

STAGES = ["build_graph", "edge_march", "floyd_warshall", "vertex_light", "diffuse", "splat", "render"]
NOMINAL_FP32_TFLOPS = 152 * 128 * 2 * 2.070 / 1000  # GB300: SMs x FP32 lanes x 2 (FMA) x 2.07 GHz
FW_SCHEDULES = {0: "per-round launches", 1: "persistent 1 CTA/SM", 2: "persistent 2 CTA/SM",
                3: "symmetric persistent 1 CTA/SM", 4: "symmetric persistent 2 CTA/SM",
                5: "symmetric persistent 2 CTA/SM, TMA-staged update operands"}
def fw_executed_flops(ld, schedule):
    """FP32 ops (add + min per update) the solve's kernels execute for one
    ld x ld matrix: the general schedules run every (i, j, k); the symmetric
    ones the 128-tiles on and above the diagonal, the strip blocks and the
    panel items of each of the nt = ld / 64 rounds."""
    if schedule < 3:
        return 2.0 * ld ** 3
    nt, nu = ld // 64, ld // 128
    tiles = nt * nu * (nu + 1) // 2 * 128 * 128 * 64
    strips = (nt - 1) * (nt - 1) * 64 ** 3
    panels = (1 + nt * (nt - 1)) * 64 ** 3
    return 2.0 * (tiles + strips + panels)


FW_KERNELS = {0: "k_fw_update+k_fw_panels", 1: "k_fw_persistent", 2: "k_fw_persistent",
              3: "k_fw_persistent_sym+k_fw_mirror", 4: "k_fw_persistent_sym+k_fw_mirror",
              5: "k_fw_persistent_sym<tma>+k_fw_mirror"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="the 128^3 / 1024-point / 256^2 case instead")
    ap.add_argument("--image", type=int, default=0, help="override the square image size (profiling runs)")
    ap.add_argument("--spp", type=int, default=0, help="override the samples per pixel (profiling runs)")
    ap.add_argument("--res", type=int, default=0, help="override the production grid resolution (profiling runs)")
    ap.add_argument("--serving", type=int, default=200, help="requests in the serving measurement (0: skip)")
    ap.add_argument("--rates", default="50", help="Poisson arrival rates of the serving stream (req/s, comma "
                                                  "separated; the full sweep is 1,5,10,25,50)")
    ap.add_argument("--batched", type=int, default=1, help="run the 64-graph batched measurement (0: skip)")
    ap.add_argument("--fw-schedule", type=int, default=-1,
                    help="pin the Floyd-Warshall schedule (0-5; -1: autotuned). Profiling runs pin the "
                         "schedule the autotuner picks without a profiler, whose per-launch overhead "
                         "distorts the trial timings")
    ap.add_argument("--ref-iters", type=int, default=500,
                    help="LightGraph iterations of the reference-scale pipeline measurement (0: skip)")
    return ap.parse_args()


def run_reference_scale(iterations: int, local: int, cpu: bool):
    """The reference's own pipeline at its own scale (its explosion scene's
    -iter 500): dart throwing of every iteration's points on the GPU, graph
    build, edge march, batched Floyd-Warshall, vertex light, diffusion, one
    splat of all points and the render, timed stage by stage (one warm-up
    pass, then one timed pass)."""
    import time
    import torch
    from lightgraph_gb300 import Context, scenes
    from lightgraph_gb300.lightgraph import scatter_opts
    sc = scenes.reference_scale(iterations)
    ctx = Context(local)
    scenes.load_into(ctx, sc)
    opts = scatter_opts()
    ms = {}
    for rep in range(2):
        t = {}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cnt = ctx.scatter_graphs(0, iterations, sc.max_connect, opts)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ctx.solve_graphs(want=False)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        ctx.splat(0.0)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        ctx.lib.lg_render(ctx.h, __import__("ctypes").byref(sc.opts.camera_c()), None, None, None, None)
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        ms = {"scatter_points_and_graph_build": (t1 - t0) * 1e3, "lightgraph_solve": (t2 - t1) * 1e3,
              "splat": (t3 - t2) * 1e3, "render": (t4 - t3) * 1e3, "frame": (t4 - t0) * 1e3}
    out = {"workload": f"{iterations} LightGraph iterations from dart throwing (1M candidates each, "
                       f"~750 points kept), production 512^3 cumulus, dir + 3-sample env light, "
                       f"{sc.opts.width}x{sc.opts.height} at {sc.opts.samples} spp",
           "points": int(cnt.sum()), "points_per_iteration": [int(cnt.min()), int(cnt.max())],
           "ms": {k: round(v, 3) for k, v in ms.items()},
           "timing": "host wall clock around each stage with a device synchronize, second of two passes"}
    if cpu:
        from oracle import pyoracle as po
        n_cpu = 16
        t0 = time.perf_counter()
        po.scatter_points(sc.density, opts, 0, n_cpu)
        dt = (time.perf_counter() - t0) * 1e3
        out["cpu_scatter_points"] = {"ms_per_frame": dt * iterations / n_cpu,
                                     "sample": f"{n_cpu} iterations scaled x{iterations / n_cpu:g}",
                                     "cores": int(po.load().lgo_threads()), "kind": "port"}
    ctx.close()
    return out


def run_batched_graphs(local: int):
    """Many graphs of uneven size in one solve: 64 graphs, N log-uniform in
    [256, 4096], each solve's Floyd-Warshall in one persistent launch (or per
    round, whichever the autotuner picks), timed with CUDA events over the
    whole LightGraph stage (graph build, edge march, Floyd-Warshall, vertex
    light, diffusion) plus the splat, after one warm-up pass."""
    import ctypes as C
    import torch
    from lightgraph_gb300 import Context, scenes
    sc = scenes.batched_graphs()
    ctx = Context(local)
    scenes.load_into(ctx, sc)
    lib = ctx.lib
    stream = torch.cuda.ExternalStream(ctx.stream)
    ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    ctx.solve_graphs(want=False)
    ctx.splat(0.0)
    torch.cuda.synchronize()
    lib.lg_set_profiling(ctx.h, 1)
    reps = 3
    buf = (C.c_double * len(STAGES))()
    stage = np.zeros(len(STAGES))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        lib.lg_frame_device(ctx.h, sc.max_connect, C.c_double(0.0), C.byref(sc.opts.camera_c()))
        if lib.lg_stage_times(ctx.h, buf, len(STAGES)) == 0:
            stage += np.array(buf[:])
    ev1.record(stream)
    torch.cuda.synchronize()
    lib.lg_set_profiling(ctx.h, 0)
    stage /= reps
    # the same frame captured once as a CUDA graph and replayed
    ctx.set_graph_mode(True)
    for _ in range(2):  # run + capture, then a replay
        lib.lg_frame_device(ctx.h, sc.max_connect, C.c_double(0.0), C.byref(sc.opts.camera_c()))
    torch.cuda.synchronize()
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record(stream)
    for _ in range(reps):
        lib.lg_frame_device(ctx.h, sc.max_connect, C.c_double(0.0), C.byref(sc.opts.camera_c()))
    ev3.record(stream)
    torch.cuda.synchronize()
    ctx.set_graph_mode(False)
    sched, tuned = ctx.fw_schedule()
    lds = [(len(p) + 127) // 128 * 128 for p in sc.points]
    flops = sum(2.0 * ld ** 3 for ld in lds)
    fw_ms = float(stage[2])
    out = {"workload": "64 LightGraphs, N log-uniform in [256, 4096] (seed 3), one 256^3 cumulus, radius 0.15, "
                       "256^2 at 1 spp", "points": int(sum(len(p) for p in sc.points)),
           "sizes": [int(min(len(p) for p in sc.points)), int(max(len(p) for p in sc.points))],
           "frame_ms": ev0.elapsed_time(ev1) / reps,
           "frame_ms_graph_replay": ev2.elapsed_time(ev3) / reps,
           "stages_ms": {k: round(float(v), 4) for k, v in zip(STAGES, stage)},
           "fw": {"schedule": FW_SCHEDULES.get(sched, str(sched)),
                  "autotuner_ms": [round(x, 4) for x in tuned], "tflops": flops / (fw_ms * 1e-3) / 1e12,
                  "frac_of_nominal_fp32": flops / (fw_ms * 1e-3) / 1e12 / NOMINAL_FP32_TFLOPS},
           "timing": "CUDA events on the frame stream, frames through lg_frame_device (graph build to render); "
                     "frame_ms with per-stage events, frame_ms_graph_replay as one captured CUDA graph"}
    ctx.close()
    return out


def run_serving(n: int, rates):
    """The mixed request stream (4 volumes 64^3..512^3, 512..8192 points,
    128^2..1024^2 at 1-4 spp, 1-3 lights plus an environment light on a
    quarter of the requests, seed 4). The same n requests are
      * rendered each alone on an idle server (single-request latency);
      * submitted all at once (capacity) to the batched server (8 slots,
        volumes resident, path solves of requests in flight sharing
        Floyd-Warshall launches), to the same server with every request
        solving its paths alone, to a one-slot resident server, and through the
        plain drop-in path (one request at a time: volume load, then
        lg_render_frame; Floyd-Warshall on the server's fixed schedule, the
        load timed apart);
      * replayed as a Poisson stream at each rate against the batched server
        (p50/p99 latency, renders/s, p99 over the alone p99)."""
    from lightgraph_gb300 import serve
    vs = serve.make_volumes(None)
    out = {"stream": f"{n} requests, Poisson arrivals, seed 4, volumes 64^3-512^3, 512-8192 points, "
                     "128^2-1024^2 at 1-4 spp, 1-3 lights, a 2-sample env light on a quarter of them"}

    def server(slots, solo_paths=False):
        srv = serve.Server(max_inflight=slots, solo_paths=solo_paths)
        vs.ids = [srv.add_volume(g) for g in vs.grids]
        return srv

    srv = server(1)
    lat = []
    for _, req in serve.request_stream(vs, n, 1.0, seed=4):
        _, _, l = srv.wait(srv.submit(req), -1, False)
        lat.append(l / 1e3)
    srv.close()
    out["alone_p50_ms"] = float(np.percentile(lat, 50))
    out["alone_p99_ms"] = float(np.percentile(lat, 99))
    cap = {}
    for label, slots, solo in (("batched_8_slots", 8, False), ("batched_8_slots_solo_paths", 8, True),
                               ("resident_1_slot", 1, True)):
        srv = server(slots, solo)
        cap[label], _ = serve.run_stream(srv, serve.request_stream(vs, n, 1.0, seed=4), realtime=False)
        srv.close()
    cap["plain_fixed_schedule"] = serve.run_standalone(vs, serve.request_stream(vs, n, 1.0, seed=4))
    b = cap["batched_8_slots"]["renders_per_s"]
    cap["batched_over_resident_1_slot"] = b / cap["resident_1_slot"]["renders_per_s"]
    cap["shared_paths_over_solo_paths"] = b / cap["batched_8_slots_solo_paths"]["renders_per_s"]
    cap["batched_over_plain"] = b / cap["plain_fixed_schedule"]["renders_per_s"]
    cap["batched_over_plain_without_upload"] = b / cap["plain_fixed_schedule"]["renders_per_s_without_upload"]
    out["capacity"] = cap
    sweep = []
    for rate in rates:
        srv = server(8)
        st, _ = serve.run_stream(srv, serve.request_stream(vs, n, rate, seed=4), realtime=True)
        srv.close()
        st["rate_req_per_s"] = rate
        st["p99_over_alone_p99"] = st["p99_ms"] / out["alone_p99_ms"]
        sweep.append(st)
    out["rates"] = sweep
    return out


def job_time_ms(t_ms: float, world: int, device: str = "cuda") -> float:
    """The job's time over N replica ranks: the maximum of the ranks' times
    (every rank runs the same number of frames)."""
    if world <= 1:
        return t_ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([t_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_scene(small: bool, image: int = 0, spp: int = 0, res: int = 0):
    from lightgraph_gb300 import scenes
    sc = scenes.small() if small else (scenes.production(res=res) if res > 0 else scenes.production())
    if image > 0:
        sc.opts.width = sc.opts.height = image
    if spp > 0:
        sc.opts.samples = spp
    return sc


def workload_config(sc, small):
    o = sc.opts
    res = sc.info["res"]
    return {"workload": ("small 128^3 sphere-fBm" if small else f"production {res}^3 sparse cumulus") +
            f", {len(sc.points[0])}-point LightGraph, {o.width}x{o.height} at {o.samples} spp",
            "grid": f"{sc.info['res']}^3, voxel {sc.info['voxel']:.5g}, active voxels {sc.info['active_voxels']}",
            "graph_points": len(sc.points[0]), "connect_radius": sc.radius[0], "max_connect": sc.max_connect,
            "image": [o.width, o.height], "spp": o.samples, "lights": [l.spec for l in sc.lights],
            "steps_per_frame": list(o.step), "precision": "fp32 grids, fp32 math",
            "l2": "inputs larger than L2 (density cell records: 32 B per voxel, active leaves ~620 MB at 512^3 "
                  "> 129 MB L2), no flush" if not small else
                  "small case: grid fits L2",
            "parallelism": "replicas (independent frames per GPU)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_traffic(name: str):
    """dram bytes per launch of a kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("dram_bytes_per_frame_launch:"):
                    return float(line.split(":", 1)[1].strip())
    except Exception:
        pass
    return None


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (the reference's loops in FP64, OpenMP) on a sample
# ---------------------------------------------------------------------------

FW_WINDOWS = 8        # Floyd-Warshall: windows of consecutive rounds, spread over the solve
SAMPLE_FRACTION = 32  # 1/32 of the Floyd-Warshall rounds and 1/32 of the image rows are timed


class CpuFrameSample:
    """The reference's frame on the host cores, timed on a bounded sample.

    One rule, used by both the --impl reference arm and the cpu_baseline leg:
      * graph build, edge march, vertex light, diffusion and splat run whole;
      * Floyd-Warshall (floydAlgo's FP64 max-times loop, OpenMP over rows):
        FW_WINDOWS windows of n / (FW_WINDOWS * SAMPLE_FRACTION) consecutive
        rounds, centred in equal parts of the solve, each started from the
        matrix as it stands at that round, scaled x SAMPLE_FRACTION. A round's
        cost depends on how far the matrix has filled in, so a prefix of
        rounds would under-count it. The states at the window starts are
        reached once, untimed, by FP32 min-plus rounds, which give floydAlgo's
        sparsity pattern after the same rounds;
      * render: the rows (r + 1/2) H / R, R = H / SAMPLE_FRACTION, in one call
        parallel over their pixels, scaled x SAMPLE_FRACTION.
    setup() does the untimed preparation once; step() times one sample.
    calibrate() measures, against a whole frame timed in the same run, the
    ratio of each sampled stage's whole-frame time to its scaled sample
    (rows rendered apart lose the cache reuse neighbouring rows get in a
    whole frame); later steps multiply the sampled stages by it."""

    def __init__(self, sc):
        self.sc = sc
        self.factors = {}

    def setup(self):
        import ctypes as C
        from oracle import pyoracle as po
        sc = self.sc
        self.po = po
        lib = self.lib = po.load()
        lib.lgo_fw_maxtimes_rounds.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int]
        lib.lgo_fw_minplus_f32_rounds.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int]
        lib.lgo_transmittance_of.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
        self.o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights, temperature=sc.temperature,
                           env_map=sc.env_map)
        self.pts = sc.points[0]
        n = self.n = len(self.pts)
        adj, _ = self.o.build_graph(self.pts, sc.radius_sq[0], sc.max_connect)
        _, S = self.o.march_edges(self.pts, adj, want_T=False)
        self.ext = np.ascontiguousarray(sc.shader.getExtinction(), np.float64)
        self.K = max(1, n // (FW_WINDOWS * SAMPLE_FRACTION))
        part = n / FW_WINDOWS
        self.k0 = [min(n - self.K, max(0, int((w + 0.5) * part - self.K / 2))) for w in range(FW_WINDOWS)]
        state = np.ascontiguousarray(S, np.float32)
        self.states, k = [], 0
        for k0 in self.k0:
            lib.lgo_fw_minplus_f32_rounds(n, state.ctypes.data, k, k0)
            k = k0
            self.states.append(state.copy())
        lib.lgo_fw_minplus_f32_rounds(n, state.ctypes.data, k, n)
        np.fill_diagonal(state, 0.0)
        self.T_solved = self._transmittance(state)
        self.T_window = np.empty((n, n, 3))
        H = sc.opts.height
        R = max(1, H // SAMPLE_FRACTION)
        self.rows = np.ascontiguousarray([min(H - 1, int((r + 0.5) * H / R)) for r in range(R)], np.int32)
        self.row_scale = H / R
        self.fw_scale = n / (FW_WINDOWS * self.K)
        return self

    def _transmittance(self, S, out=None):
        n = S.shape[0]
        out = np.empty((n, n, 3)) if out is None else out
        S64 = np.ascontiguousarray(S, np.float64)
        self.lib.lgo_transmittance_of(n * n, S64.ctypes.data, self.ext.ctypes.data, out.ctypes.data)
        return out

    def calibrate(self, full_stages):
        """Per sampled stage, whole-frame ms / scaled sample ms, from the mean
        of two warm samples against the whole frame's stage times."""
        self.factors = {}
        dets = [self.step()[1] for _ in range(2)]
        for k in ("floyd_warshall", "render"):
            self.factors[k] = full_stages[k] / (0.5 * (dets[0][k] + dets[1][k]))
        return self.factors

    def describe(self):
        d = (f"build/march/light/diffuse/splat whole; Floyd-Warshall {FW_WINDOWS} windows of {self.K} rounds "
             f"spread over {self.n} (each from the matrix's state at its round) scaled x{self.fw_scale:g}; "
             f"render rows (r+1/2)H/{len(self.rows)} ({len(self.rows)} of {self.sc.opts.height}) in one "
             f"pixel-parallel call scaled x{self.row_scale:g}")
        if self.factors:
            d += ("; both sampled stages then scaled by their whole-frame/sample ratio measured once in this run "
                  f"(Floyd-Warshall x{self.factors['floyd_warshall']:.3f}, render x{self.factors['render']:.3f})")
        return d

    def step(self):
        """One timed sample: (ms per frame, per-stage ms)."""
        import ctypes as C
        o, sc, pts, n, lib = self.o, self.sc, self.pts, self.n, self.lib
        det = {}
        t = time.perf_counter()
        adj, _ = o.build_graph(pts, sc.radius_sq[0], sc.max_connect)
        det["build_graph"] = (time.perf_counter() - t) * 1e3
        t = time.perf_counter()
        o.march_edges(pts, adj)
        det["edge_march"] = (time.perf_counter() - t) * 1e3
        fw = 0.0
        for k0, st in zip(self.k0, self.states):
            self._transmittance(st, self.T_window)
            t = time.perf_counter()
            lib.lgo_fw_maxtimes_rounds(n, self.T_window.ctypes.data, k0, k0 + self.K)
            fw += time.perf_counter() - t
        det["floyd_warshall"] = fw * 1e3 * self.fw_scale * self.factors.get("floyd_warshall", 1.0)
        t = time.perf_counter()
        L = o.vertex_light(pts)
        det["vertex_light"] = (time.perf_counter() - t) * 1e3
        t = time.perf_counter()
        D = o.diffuse(self.T_solved, L)
        det["diffuse"] = (time.perf_counter() - t) * 1e3
        t = time.perf_counter()
        lo, dims, sg, _ = o.splat(pts, D)
        det["splat"] = (time.perf_counter() - t) * 1e3
        W, H = sc.opts.width, sc.opts.height
        films = [np.zeros((H, W, 4), np.float32) for _ in range(4)]
        vals = np.ascontiguousarray(sg, np.float32)
        cam = sc.opts.camera_c()
        lib.lgo_render_rows.argtypes = None
        t = time.perf_counter()
        lib.lgo_render_rows(C.byref(o.dens), C.byref(o.temp) if o.temp else None, C.byref(o.shader),
                            C.byref(o.settings), o.lights, o.n_lights, C.byref(o.env) if o.env else None,
                            C.byref(cam), (C.c_int32 * 3)(*lo), (C.c_int32 * 3)(*dims),
                            C.c_double(sc.density.voxel_size * sc.opts.scatterGridResFactor),
                            C.c_void_p(vals.ctypes.data), C.c_void_p(self.rows.ctypes.data), C.c_int(len(self.rows)),
                            *[C.c_void_p(f.ctypes.data) for f in films], None)
        det["render"] = (time.perf_counter() - t) * 1e3 * self.row_scale * self.factors.get("render", 1.0)
        return sum(det.values()), det


def cpu_full_frame(sc):
    """The whole frame on the host cores, nothing sampled: FP64 max-times
    Floyd-Warshall over every round, every image row. Returns (ms, stages)."""
    from oracle import pyoracle as po
    o = po.Oracle(sc.density, sc.shader, sc.opts, sc.lights, temperature=sc.temperature, env_map=sc.env_map)
    pts = sc.points[0]
    det = {}

    def timed(name, fn, *a):
        t = time.perf_counter()
        r = fn(*a)
        det[name] = (time.perf_counter() - t) * 1e3
        return r
    adj, _ = timed("build_graph", o.build_graph, pts, sc.radius_sq[0], sc.max_connect)
    T, _ = timed("edge_march", o.march_edges, pts, adj)
    Tsol = timed("floyd_warshall", o.fw_maxtimes, T)
    del T
    L = timed("vertex_light", o.vertex_light, pts)
    D = timed("diffuse", o.diffuse, Tsol, L)
    del Tsol
    lo, dims, sg, _ = timed("splat", o.splat, pts, D)
    timed("render", o.render, (lo, dims, sg))
    return sum(det.values()), det


def sampler_error(smp, full_ms):
    """The uncalibrated sampling rule against the whole frame of the same
    workload timed complete on the host cores: one sample after a warm-up."""
    saved, smp.factors = smp.factors, {}
    smp.step()
    est = smp.step()[0]
    smp.factors = saved
    return {"full_frame_ms": full_ms, "sampled_estimate_ms": est, "relative_error": (est - full_ms) / full_ms}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    sc = make_scene(args.small, args.image, args.spp, args.res)
    full, full_det = cpu_full_frame(sc)
    smp = CpuFrameSample(sc).setup()
    check = sampler_error(smp, full)
    check["factors"] = smp.calibrate(full_det)
    check["full_frame_stages_ms"] = {k: round(x, 3) for k, x in full_det.items()}
    for _ in range(args.warmup):
        smp.step()
    vals, det_acc = [], {}
    for _ in range(args.steps):
        v, det = smp.step()
        vals.append(v)
        for k, x in det.items():
            det_acc[k] = det_acc.get(k, 0.0) + x / args.steps
    value = float(np.mean(vals))
    threads = smp.o.threads()
    line = {"metric": "ms/frame", "value": value, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_config(sc, args.small),
            "cpu_baseline": {"value": value, "unit": "ms/frame", "cores": threads, "kind": "port",
                             "sample": smp.describe(), "stages_ms": {k: round(x, 3) for k, x in det_acc.items()},
                             "sampler_check": check},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args):
    import torch
    import torch.distributed as dist
    from lightgraph_gb300 import Context, scenes

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    sc = make_scene(args.small, args.image, args.spp, args.res)
    ctx = Context(local)
    scenes.load_into(ctx, sc)
    ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
    if args.fw_schedule >= 0:
        ctx.set_fw_schedule(args.fw_schedule)
    lib = ctx.lib
    stream = torch.cuda.ExternalStream(ctx.stream)

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(max(3, args.warmup)):
        ctx.frame_device(sc.opts, sc.max_connect)
    torch.cuda.synchronize()
    prim, shad = ctx.render_stats()
    tasks_per_frame = ctx.shading_tasks()

    # timed region: K frames, grids and points resident
    lib.lg_set_profiling(ctx.h, 1)
    import ctypes as C
    stage_ms = np.zeros(len(STAGES))
    launches0 = ctx.kernel_launches()
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    buf = (C.c_double * len(STAGES))()
    wbuf = (C.c_double * 5)()
    wave_ms = np.zeros(5)
    for _ in range(args.steps):
        ctx.frame_device(sc.opts, sc.max_connect)
        if lib.lg_stage_times(ctx.h, buf, len(STAGES)) == 0:
            stage_ms += np.array(buf[:])
        if lib.lg_render_wave_times(ctx.h, wbuf) == 0:
            wave_ms += np.array(wbuf[:])
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = ctx.kernel_launches() - launches0
    lib.lg_set_profiling(ctx.h, 0)
    t_ms = job_time_ms(ev0.elapsed_time(ev1), world)
    ms_per_step = t_ms / args.steps
    value = ms_per_step / world
    stage_ms /= args.steps
    wave_ms /= args.steps

    # e2e through the C ABI from pinned host memory
    pts = sc.points[0]
    n = len(pts)
    W, H = sc.opts.width, sc.opts.height
    pin_pts = torch.from_numpy(np.ascontiguousarray(pts)).pin_memory()
    offs = torch.tensor([0, n], dtype=torch.int64).pin_memory()
    r2 = torch.tensor([float(sc.radius_sq[0])], dtype=torch.float32).pin_memory()
    films = [torch.empty((H, W, 4), dtype=torch.float32).pin_memory() for _ in range(4)]
    cam = sc.opts.camera_c()
    for _ in range(1):
        lib.lg_render_frame(ctx.h, 1, pin_pts.data_ptr(), offs.data_ptr(), r2.data_ptr(), sc.max_connect, 0.0,
                            C.byref(cam), *[f.data_ptr() for f in films])
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = lib.lg_render_frame(ctx.h, 1, pin_pts.data_ptr(), offs.data_ptr(), r2.data_ptr(), sc.max_connect, 0.0,
                                 C.byref(cam), *[f.data_ptr() for f in films])
        if st != 0:
            raise RuntimeError(lib.lg_last_error(ctx.h).decode())
    e2e_ms = job_time_ms((time.perf_counter() - t0) * 1e3 / args.steps, world)
    e2e_value = e2e_ms / world
    h2d = pin_pts.numel() * 4 + offs.numel() * 8 + r2.numel() * 4
    d2h = sum(f.numel() * 4 for f in films)

    peaks, peak_kind = measured_peaks()
    # dominant kernel: k_shadow (the shadow-ray wave of the render). Its
    # algorithmic bytes per launch: 8 taps x 4 B per shadow density sample
    # plus, per shading sample and light, the 4 B order entry and 32 B task
    # read and the 16 B result write.
    n_lights = len(sc.lights)
    shadow_ms = wave_ms[3]
    shadow_bytes = shad * 32.0 + tasks_per_frame * n_lights * 52.0
    achieved = shadow_bytes / (shadow_ms * 1e-3) / 1e9
    render_bytes = (prim + shad) * 32.0 + W * H * 64.0
    render_gbs = render_bytes / (stage_ms[6] * 1e-3) / 1e9
    ld = (len(pts) + 127) // 128 * 128  # the solve runs on the 128-padded matrix
    fw_sched, fw_tuned = ctx.fw_schedule()
    fw_flops = 2.0 * ld ** 3
    fw_tflops = fw_flops / (stage_ms[2] * 1e-3) / 1e12
    fw_exec = fw_executed_flops(ld, fw_sched)
    fw_ceiling = ctx.fw_inner_loop_rate()
    line = {
        "metric": "ms/frame", "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm volumes, uniform interior points)",
        "config": workload_config(sc, args.small),
        "e2e": {"value": e2e_value, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clk,
        "stages_ms": {k: round(float(v), 4) for k, v in zip(STAGES, stage_ms)},
        "roofline": {"kernel": "k_shadow", "bound": "hbm", "achieved": achieved,
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved / peaks.get("hbm_gbs"), "peak_kind": peak_kind + " (burst copy)",
                     "traffic": profile_traffic("k_shadow_production.txt"),
                     "algorithmic_bytes": shadow_bytes, "launch_ms": shadow_ms,
                     "samples": {"primary": prim, "shadow": shad, "shading_tasks": tasks_per_frame}},
        "render_waves_ms": {"count_scan": wave_ms[0], "primary": wave_ms[1], "ray_order": wave_ms[2],
                            "shadow": wave_ms[3], "resolve": wave_ms[4]},
        "render_stage": {"ms": float(stage_ms[6]), "algorithmic_bytes": render_bytes, "achieved_gbs": render_gbs,
                         "frac": render_gbs / peaks.get("hbm_gbs")},
        "fw_roofline": {"kernel": FW_KERNELS.get(fw_sched, "?"),
                        "bound": "fp32_alu", "n": int(ld),
                        "achieved": fw_tflops, "unit": "TFLOP/s", "peak": NOMINAL_FP32_TFLOPS,
                        "peak_kind": "nominal (152 SMs x 128 lanes x 2 x 2.07 GHz)",
                        "frac": fw_tflops / NOMINAL_FP32_TFLOPS,
                        "schedule": FW_SCHEDULES.get(fw_sched, str(fw_sched)),
                        "autotuner_ms": [round(x, 4) for x in fw_tuned],
                        "executed_tflops": fw_exec / (stage_ms[2] * 1e-3) / 1e12,
                        "inner_loop_ceiling_tflops": fw_ceiling,
                        "executed_frac_of_inner_loop_ceiling": fw_exec / (stage_ms[2] * 1e-3) / 1e12 / fw_ceiling},
    }
    if rank == 0 and args.serving > 0:
        line["serving"] = run_serving(args.serving, [float(r) for r in args.rates.split(",") if r])
    if rank == 0 and world == 1 and args.ref_iters > 0 and not args.small:
        line["reference_scale"] = run_reference_scale(args.ref_iters, local, not args.no_cpu_baseline)
    if rank == 0 and world == 1 and args.batched and not args.small:
        line["batched_graphs"] = run_batched_graphs(local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the whole frame, measured (no sampling), and the sampling rule the
        # --impl reference arm uses checked against it
        from oracle import pyoracle as po
        full, det = cpu_full_frame(sc)
        smp = CpuFrameSample(sc).setup()
        line["cpu_baseline"] = {"value": full, "unit": "ms/frame", "cores": int(po.load().lgo_threads()),
                                "kind": "port", "sample": "the whole frame, timed once (nothing sampled or scaled)",
                                "stages_ms": {k: round(x, 3) for k, x in det.items()},
                                "sampler_check": sampler_error(smp, full)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
