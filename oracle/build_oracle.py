#!/usr/bin/env python3
"""Build recipe of the oracle restatement: oracle/_build/liboracle.so, and of the synthetic
inputs' generator for the CPU side: oracle/_build/libscenegen.so.

TEST INFRASTRUCTURE (oracle). g++ -O2 -std=c++17 -ffp-contract=off (no fused
multiply-add: every float operation is the one written) -fopenmp. Portable flags only, so
the same recipe builds on x86-64 and aarch64 hosts.

libscenegen.so is the seeded scene and camera generator that defines the workloads (the
library's csrc/host_scene.cpp, compiled here on its own): the CPU reference arm of the benchmark
builds its scene arrays and cameras with it, so that it loads the oracle's libraries only.
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SOURCES = ["gris_oracle.cpp", "converged_fp64.cpp"]


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    h = hashlib.sha256()
    for f in SOURCES + ["detmath.h", os.path.basename(__file__)]:
        with open(os.path.join(HERE, f), "rb") as fh:
            h.update(fh.read())
    stamp = os.path.join(OUT, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB] + [os.path.join(HERE, s) for s in SOURCES]
    if subprocess.call(cmd) != 0:
        raise RuntimeError("oracle build failed")
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    return LIB


SCENEGEN = os.path.join(OUT, "libscenegen.so")
SCENEGEN_SRC = os.path.join(os.path.dirname(HERE), "vulkan-restir-pt_gb300", "csrc", "host_scene.cpp")


def build_scenegen(force=False):
    os.makedirs(OUT, exist_ok=True)
    csrc = os.path.dirname(SCENEGEN_SRC)
    h = hashlib.sha256()
    for f in ("host_scene.cpp", "detmath.h", "grisrt_internal.h", os.path.join("..", "..", "include", "grisrt.h")):
        with open(os.path.join(csrc, f), "rb") as fh:
            h.update(fh.read())
    with open(__file__, "rb") as fh:
        h.update(fh.read())
    stamp = os.path.join(OUT, "stamp_scenegen")
    if not force and os.path.exists(SCENEGEN) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return SCENEGEN
    cxx = os.environ.get("CXX", "g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", cuda_inc, "-o", SCENEGEN, SCENEGEN_SRC]
    if subprocess.call(cmd) != 0:
        raise RuntimeError("scene generator build failed")
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    return SCENEGEN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_scenegen(force="--force" in sys.argv))
