#!/usr/bin/env python3
"""Generates the golden vectors in tests/golden/ from the reference's own shader code compiled
as C++ (oracle/_ref, built by oracle/ref/make_ref.py where the reference sources are present):
the GRIS pass (libgrisref.so) and, in the di_*.npz files, the ReSTIR DI pass (libdiref.so, on the
G-buffer of libgrisref.so).

For each case the file stores the scene-array hash, the cameras and settings used, the ray
counts, and per frame the SHA-256 digest of every buffer (G-buffer, motion, reservoirs,
temporary reservoirs, output) plus, for the small cases, full copies of the reservoirs and the
output radiance (for diagnostics).
Usage: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "vulkan-restir-pt_gb300"))
sys.path.insert(0, REPO)

import grisrt as G                      # noqa: E402
from oracle import pyoracle as O        # noqa: E402

BUFFERS = ("dn", "am", "mv", "resv", "temp", "out")
# name: (kind, grid, spheres, W, H, frames, settings, store full arrays)
CASES = {
    "box_32x32_c1": (0, 0, 0, 32, 32, 3, dict(maxDepth=3, spatialRadius=30.0), True),
    "terrain_24x20_d8": (1, 24, 12, 24, 20, 2, dict(maxDepth=8, spatialRadius=30.0), True),
    "glossy_24x20_d8": (2, 24, 12, 24, 20, 2, dict(maxDepth=8), True),
    "box_256x256_c1_8frames": (0, 0, 0, 256, 256, 8, dict(maxDepth=3, spatialRadius=30.0), False),
    "terrain_32x24_9nb_cap3": (1, 32, 40, 32, 24, 3, dict(maxDepth=6, spatialNeighbors=9, cap=3), False),
}
DI_BUFFERS = ("resv", "temp", "out")
# name: (kind, grid, spheres, W, H, frames, DI settings)
DI_CASES = {
    "di_box_32x32_temporal": (0, 0, 0, 32, 32, 3, dict(temporalReuse=True)),
    "di_box_32x24_replay_both": (0, 0, 0, 32, 24, 2, dict(shiftType=1, sampleType=2, temporalReuse=True)),
    "di_terrain_24x20_both": (1, 24, 12, 24, 20, 2, dict(sampleType=2, temporalReuse=True)),
}


def scene_hash(hs):
    h = hashlib.sha256()
    for a in hs.arrays():
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make(name):
    kind, grid, spheres, W, H, frames, kw, full = CASES[name]
    G.load()
    hs = G.HostScene(kind, seed=3, grid=grid, spheres=spheres)
    cams, prevs = G.sequence_cameras(hs, frames, W, H, seed=21)
    st = G.Settings.make(**kw)
    ref = O.reference()
    ref.set_scene(hs)
    ref.read_counters(reset=True)
    res = O.run_sequence(ref, cams, prevs, st, W, H)
    cnt = ref.read_counters(reset=True)
    out = {"scene_sha256": np.array(scene_hash(hs)), "settings": np.frombuffer(bytes(memoryview(st)), np.uint8),
           "cams": np.stack([np.frombuffer(c.tobytes(), np.uint8) for c in cams]),
           "prevs": np.stack([np.frombuffer(c.tobytes(), np.uint8) for c in prevs]),
           "counters": np.array(cnt[:3], np.uint64), "meta": np.array([kind, grid, spheres, W, H, frames], np.int64)}
    for f in range(frames):
        for k in BUFFERS:
            if full and k in ("resv", "out"):
                out["%s_%d" % (k, f)] = res[f][k]
            out["%s_%d_sha256" % (k, f)] = np.array(digest(res[f][k]))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path


def make_di(name):
    kind, grid, spheres, W, H, frames, kw = DI_CASES[name]
    G.load()
    hs = G.HostScene(kind, seed=3, grid=grid, spheres=spheres)
    cams, prevs = G.sequence_cameras(hs, frames, W, H, seed=23)
    di = G.DISettings.make(**kw)
    gref, dref = O.reference(), O.reference_di()
    gref.set_scene(hs)
    dref.set_scene(hs)
    dref.read_counters(reset=True)
    res = O.run_di_sequence(gref, dref, cams, prevs, di, W, H)
    cnt = dref.read_counters(reset=True)
    out = {"scene_sha256": np.array(scene_hash(hs)), "di_settings": np.frombuffer(bytes(memoryview(di)), np.uint8),
           "cams": np.stack([np.frombuffer(c.tobytes(), np.uint8) for c in cams]),
           "prevs": np.stack([np.frombuffer(c.tobytes(), np.uint8) for c in prevs]),
           "counters": np.array(cnt[:2], np.uint64), "meta": np.array([kind, grid, spheres, W, H, frames], np.int64)}
    for f in range(frames):
        for k in DI_BUFFERS:
            out["%s_%d" % (k, f)] = res[f][k]
            out["%s_%d_sha256" % (k, f)] = np.array(digest(res[f][k]))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    return path


# visual regression: name -> (kind, grid, spheres, W, H, frames, GRIS settings, DI settings)
PNG_CASES = {
    "post_box_48x32": (0, 0, 0, 48, 32, 4, dict(maxDepth=4), dict(sampleType=2, temporalReuse=True)),
}


def make_png(name):
    """The renderer's frame with both passes (GRIS and ReSTIR DI from the reference's shaders run
    as C++), presented by the reference's post_proc.frag run as C++ (filmic, gamma, UNORM8) and
    written with the library's PNG writer; the inputs go into <name>.npz beside the image."""
    kind, grid, spheres, W, H, frames, kw, dkw = PNG_CASES[name]
    G.load()
    hs = G.HostScene(kind, seed=3, grid=grid, spheres=spheres)
    cams, prevs = G.sequence_cameras(hs, frames, W, H, seed=29)
    st, di, post = G.Settings.make(**kw), G.DISettings.make(**dkw), G.PostSettings.make()
    gref, dref = O.reference(), O.reference_di()
    gref.set_scene(hs)
    dref.set_scene(hs)
    ind = O.run_sequence(gref, cams, prevs, st, W, H, record=("out",))[-1]["out"]
    dirr = O.run_di_sequence(gref, dref, cams, prevs, di, W, H, record=("out",))[-1]["out"]
    _, rgba = O.post_process(W, H, dirr, ind, post, reference=True)
    G.write_png(os.path.join(HERE, name + ".png"), rgba, W, H)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), scene_sha256=np.array(scene_hash(hs)),
                        settings=np.frombuffer(bytes(memoryview(st)), np.uint8),
                        di_settings=np.frombuffer(bytes(memoryview(di)), np.uint8),
                        post_settings=np.frombuffer(bytes(memoryview(post)), np.uint8),
                        cams=np.stack([np.frombuffer(c.tobytes(), np.uint8) for c in cams]),
                        prevs=np.stack([np.frombuffer(c.tobytes(), np.uint8) for c in prevs]),
                        meta=np.array([kind, grid, spheres, W, H, frames], np.int64))
    return os.path.join(HERE, name + ".png")


if __name__ == "__main__":
    if not all(os.path.exists(p) for p in (O.REF_LIB, O.DI_REF_LIB, O.POST_REF_LIB)):
        sys.exit("oracle/_ref libraries missing: run oracle/ref/make_ref.py (needs the reference sources)")
    for n in (sys.argv[1:] or list(CASES) + list(DI_CASES) + list(PNG_CASES)):
        if n in PNG_CASES:
            print(make_png(n), os.path.getsize(os.path.join(HERE, n + ".png")))
            continue
        print(make_di(n) if n in DI_CASES else make(n), os.path.getsize(os.path.join(HERE, n + ".npz")))
