"""Build recipe for the native parts of lightgraph_gb300.

Compiles, in parallel and only when sources changed:
  * lightgraph_gb300/_build/liblightgraph_gb300.so  -- CUDA kernels for sm_103a
    (nvcc -gencode arch=compute_103a,code=sm_103a) plus the C ABI;
  * lightgraph_gb300/_build/liblightgraph_host.so   -- host-only helpers, no CUDA
    (g++ -fopenmp -ffp-contract=off): the seeded synthetic scenes, the scene
    description defaults and parsers, and the EXR reader and writer. The CPU
    baseline builds its scenes through this library alone;
  * lightgraph_gb300/_build/lightgraph              -- the command-line renderer
    (links both libraries);
  * oracle/_build/liblg_oracle.so                   -- the CPU oracle used by the
    tests and the CPU baseline (test infrastructure, never linked into the
    product library);
  * oracle/_ref/libref_randgen.so                   -- where the reference source
    tree is present, its RandGen compiled from it (oracle/build_ref.py), which
    the tests use to pin the oracle's random sequence.
No CMake; nvcc and g++ only, so the same recipe runs on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "lightgraph_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "lightgraph_gb300", "_build")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")

LIB_NAME = "liblightgraph_gb300.so"
HOST_LIB_NAME = "liblightgraph_host.so"
ORACLE_NAME = "liblg_oracle.so"

CU_SOURCES = ["lg_api.cu", "k_graph.cu", "k_march.cu", "k_fw.cu", "k_diffuse.cu", "k_splat.cu",
              "k_render.cu", "k_grid.cu", "k_dart.cu", "lg_server.cu", "lg_noalloc.cu"]
HOST_SOURCES = ["scene.cc", "lg_parse.cc", "lg_exr.cc"]
CLI_SOURCE = "cli.cc"
ORACLE_SOURCES = ["lg_oracle.cc"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FP contraction, so host arithmetic rounds the same on x86 and Arm
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]
GXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]


def lib_path() -> str:
    return os.path.join(BUILD, LIB_NAME)


def host_lib_path() -> str:
    return os.path.join(BUILD, HOST_LIB_NAME)


def oracle_path() -> str:
    return os.path.join(ORACLE_BUILD, ORACLE_NAME)


def cli_path() -> str:
    return os.path.join(BUILD, "lightgraph")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build lightgraph_gb300")


def _headers(*dirs: str) -> list[str]:
    out = []
    for d in dirs:
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                out.append(os.path.join(d, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)


def build_library(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers(CSRC, INCLUDE)
    jobs_list = []
    objs, host_objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs_list.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        host_objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs_list.append(["g++"] + GXX_FLAGS + ["-c", s, "-o", o])
    n = jobs or min(len(jobs_list), os.cpu_count() or 4) or 1
    with cf.ThreadPoolExecutor(max_workers=n) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs_list]:
            f.result()
    host = host_lib_path()
    if _stale(host, host_objs):
        _run(["g++", "-shared", "-o", host] + host_objs + ["-fopenmp"], verbose)
    lib = lib_path()
    if _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"], verbose)
    cli = cli_path()
    cli_src = os.path.join(CSRC, CLI_SOURCE)
    if _stale(cli, [cli_src, lib, host] + hdrs):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", cli, "-L" + BUILD, "-llightgraph_gb300",
              "-llightgraph_host", "-Wl,-rpath,$ORIGIN"], verbose)
    return lib


def build_oracle(verbose: bool = False) -> str:
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, s) for s in ORACLE_SOURCES]
    out = oracle_path()
    deps = srcs + _headers(ORACLE_DIR)
    if _stale(out, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-I" + ORACLE_DIR] + srcs + ["-o", out], verbose)
    return out


def build_reference_part(verbose: bool = False) -> None:
    """oracle/_ref: the part of the reference that compiles here (its RandGen),
    built by oracle/build_ref.py when the reference source tree is present
    (test infrastructure; nothing is built without the tree)."""
    _run([sys.executable, os.path.join(ORACLE_DIR, "build_ref.py")] + (["-v"] if verbose else []), verbose)


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        a = ex.submit(build_library, verbose)
        b = ex.submit(build_oracle, verbose)
        c = ex.submit(build_reference_part, verbose)
        a.result()
        b.result()
        c.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(lib_path())
    print(host_lib_path())
    print(oracle_path())
