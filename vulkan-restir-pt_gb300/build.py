#!/usr/bin/env python3
"""Build recipe of libgrisrt.so (the C-ABI library with the sm_103a kernels), in-tree.

Translation units are compiled in parallel with nvcc; device code uses
-gencode arch=compute_103a,code=sm_103a --fmad=false with IEEE division and square root,
host code -ffp-contract=off, so the float sequences written in the sources are the ones
executed. The output goes to vulkan-restir-pt_gb300/grisrt/libgrisrt.so; a stamp of the
source hashes skips the build when nothing changed.
"""
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
REPO = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "grisrt")
LIB = os.path.join(OUT_DIR, "libgrisrt.so")
BUILD = os.path.join(HERE, "_build")

CUDA_SOURCES = ["gris_kernels.cu", "di_kernels.cu", "post.cu", "noalloc.cu", "guide.cu", "guide_tc.cu", "measure.cu"]
HOST_SOURCES = ["capi.cpp", "batch.cpp", "host_scene.cpp", "bvh_build.cpp", "guide_api.cpp", "image_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stamp():
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(REPO, "include")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    with open(__file__, "rb") as fh:
        h.update(fh.read())
    return h.hexdigest()


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp_file = os.path.join(BUILD, "stamp")
    st = _stamp()
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == st:
                return LIB
    nv = nvcc()
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        cmd = [nv, "-c", os.path.join(CSRC, s), "-o", o] + ARCH + [
            "-O3", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
            "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append(subprocess.Popen(cmd))
        objs.append(o)
    for s in HOST_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        cmd = [nv, "-c", os.path.join(CSRC, s), "-o", o, "-O2", "-std=c++17",
               "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp"]
        jobs.append(subprocess.Popen(cmd))
        objs.append(o)
    rc = [j.wait() for j in jobs]
    if any(rc):
        raise RuntimeError("grisrt: compilation failed")
    link = [nv, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"]
    if subprocess.call(link) != 0:
        raise RuntimeError("grisrt: link failed")
    with open(stamp_file, "w") as f:
        f.write(st)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
