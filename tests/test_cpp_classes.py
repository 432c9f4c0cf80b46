"""The C++ class layer (include/lightgraph.hpp): the reference's LightGraph,
ScatterGrid and VolumeRender over the C ABI. tests/cpp_classes_program.cc is
built against the two libraries like any C++ caller would build it; without
a GPU its Context reports LG_ERR_NODEVICE as an exception, and on a GPU a
small frame through the classes equals, bit for bit, the same frame through
the lg_* calls made directly."""
import os
import subprocess

import pytest

from lightgraph_gb300 import build

from .conftest import has_gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_program(tmp_path) -> str:
    build.build_library()
    exe = str(tmp_path / "cpp_classes")
    cmd = ["g++", "-O1", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp_classes_program.cc"), "-o", exe, "-L" + build.BUILD,
           "-llightgraph_gb300", "-llightgraph_host", "-Wl,-rpath," + build.BUILD]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_classes_build_and_report_no_device(tmp_path):
    if has_gpu():
        pytest.skip("a GPU is present: test_classes_frame_matches_c_abi covers the classes")
    exe = compile_program(tmp_path)
    r = subprocess.run([exe, "nodevice"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("error 6"), r.stdout


@pytest.mark.gpu
def test_classes_frame_matches_c_abi(tmp_path):
    if not has_gpu():
        pytest.skip("no CUDA device")
    exe = compile_program(tmp_path)
    r = subprocess.run([exe, "frame"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("match"), r.stdout


def test_c_headers_compile_as_c99(tmp_path):
    """The C ABI's headers are plain C: a C99 caller includes them with
    strict warnings (no C++ in them, no compiler extensions)."""
    src = tmp_path / "check.c"
    src.write_text('#include "lightgraph_c.h"\n#include "lightgraph_scene.h"\n'
                   "int main(void) { lg_shader s; lg_shader_default(&s); return (int)s.ramp_n; }\n")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror",
                        "-I" + os.path.join(ROOT, "include"), "-c", str(src), "-o", str(tmp_path / "check.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
