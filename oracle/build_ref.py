"""Builds oracle/_ref/libref_randgen.so: the reference's own RandGen
(src/RandGen.h), compiled from the reference source tree where it lies, with
a C entry point (oracle/ref_randgen.cc). Test infrastructure only.

The reference's other sources include OpenVDB, OpenEXR, TBB or Boost, none of
which is available, so this is the only part of the reference that builds
here. Nothing is copied: the header is read from the reference tree at build
time; without that tree nothing is built and the tests that use it skip.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/src"
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "libref_randgen.so")


def build(verbose: bool = False) -> str | None:
    if not os.path.exists(os.path.join(REF_SRC, "RandGen.h")):
        return None
    src = os.path.join(HERE, "ref_randgen.cc")
    deps = [src, os.path.join(REF_SRC, "RandGen.h")]
    if os.path.exists(OUT) and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in deps):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + REF_SRC, src, "-o", OUT]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference RandGen build failed:\n" + r.stdout)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
