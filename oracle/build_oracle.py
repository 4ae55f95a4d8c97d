#!/usr/bin/env python3
"""Build recipe of the oracle restatement: oracle/_build/liboracle.so.

TEST INFRASTRUCTURE (oracle). g++ -O2 -std=c++17 -ffp-contract=off (no fused
multiply-add: every float operation is the one written) -fopenmp. Portable flags only, so
the same recipe builds on x86-64 and aarch64 hosts.
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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
