"""Golden vectors (tests/golden/*.npz, generated by tests/golden/make_golden.py from the
reference's shaders compiled as C++): the oracle (CPU) and the CUDA path (GPU) must reproduce
every buffer of every frame bit for bit, and the ray counts — for the GRIS pass and (di_*.npz)
for the ReSTIR DI pass."""
import glob
import hashlib
import os

import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ALL = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
FILES = [p for p in ALL if not os.path.basename(p).startswith("di_")]
DI_FILES = [p for p in ALL if os.path.basename(p).startswith("di_")]
BUFFERS = ("dn", "am", "mv", "resv", "temp", "out")
DI_BUFFERS = ("resv", "temp", "out")


def load_case(path):
    z = np.load(path)
    kind, grid, spheres, W, H, frames = [int(x) for x in z["meta"]]
    hs = G.HostScene(kind, seed=3, grid=grid, spheres=spheres)
    h = hashlib.sha256()
    for a in hs.arrays():
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(z["scene_sha256"]), "scene generator output differs from the golden scene"
    cams = [G.Camera.from_buffer_copy(bytes(c)) for c in z["cams"]]
    prevs = [G.Camera.from_buffer_copy(bytes(c)) for c in z["prevs"]]
    st = G.Settings.from_buffer_copy(bytes(z["settings"]))
    return z, hs, cams, prevs, st, W, H, frames


def check(z, results, counters, frames):
    for f in range(frames):
        for k in BUFFERS:
            got = np.ascontiguousarray(results[f][k])
            if "%s_%d" % (k, f) in z.files:
                want = z["%s_%d" % (k, f)]
                assert got.tobytes() == want.tobytes(), "frame %d %s differs from the golden vector" % (f, k)
            assert hashlib.sha256(got.tobytes()).hexdigest() == str(z["%s_%d_sha256" % (k, f)]), \
                "frame %d %s digest differs from the golden vector" % (f, k)
    assert list(counters[:3]) == [int(x) for x in z["counters"]]


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(p)[:-4] for p in FILES])
def test_oracle_reproduces_golden_vectors(path):
    z, hs, cams, prevs, st, W, H, frames = load_case(path)
    ora = O.oracle()
    ora.set_scene(hs)
    ora.read_counters(reset=True)
    res = O.run_sequence(ora, cams, prevs, st, W, H)
    check(z, res, ora.read_counters(reset=True), frames)


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(p)[:-4] for p in FILES])
def test_gpu_reproduces_golden_vectors(path):
    z, hs, cams, prevs, st, W, H, frames = load_case(path)
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    ctx.counters(reset=True)
    res = []
    for f in range(frames):
        fr.render(scene, cams[f], prevs[f], st)
        res.append({"resv": fr.download(G.BUF_RESERVOIR), "temp": fr.download(G.BUF_TEMP), "out": fr.download(G.BUF_OUTPUT),
                    "dn": fr.download(G.BUF_DEPTH_NORMAL), "am": fr.download(G.BUF_ALBEDO_MATID),
                    "mv": fr.download(G.BUF_MOTION)})
    ctx.sync()
    check(z, res, ctx.counters(reset=True), frames)
    fr.close(); scene.close(); ctx.close()


def load_di_case(path):
    z = np.load(path)
    kind, grid, spheres, W, H, frames = [int(x) for x in z["meta"]]
    hs = G.HostScene(kind, seed=3, grid=grid, spheres=spheres)
    h = hashlib.sha256()
    for a in hs.arrays():
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(z["scene_sha256"]), "scene generator output differs from the golden scene"
    cams = [G.Camera.from_buffer_copy(bytes(c)) for c in z["cams"]]
    prevs = [G.Camera.from_buffer_copy(bytes(c)) for c in z["prevs"]]
    di = G.DISettings.from_buffer_copy(bytes(z["di_settings"]))
    return z, hs, cams, prevs, di, W, H, frames


def check_di(z, results, counters, frames):
    for f in range(frames):
        for k in DI_BUFFERS:
            got = np.ascontiguousarray(results[f][k])
            assert got.tobytes() == z["%s_%d" % (k, f)].tobytes(), "frame %d DI %s differs from the golden vector" % (f, k)
    assert list(counters[:2]) == [int(x) for x in z["counters"]]


@pytest.mark.parametrize("path", DI_FILES, ids=[os.path.basename(p)[:-4] for p in DI_FILES])
def test_oracle_reproduces_di_golden_vectors(path):
    z, hs, cams, prevs, di, W, H, frames = load_di_case(path)
    ora = O.oracle()
    ora.set_scene(hs)
    ora.read_counters(reset=True)
    res = O.run_di_sequence(ora, ora, cams, prevs, di, W, H)
    check_di(z, res, ora.read_counters(reset=True), frames)


@pytest.mark.gpu
@pytest.mark.parametrize("path", DI_FILES, ids=[os.path.basename(p)[:-4] for p in DI_FILES])
def test_gpu_reproduces_di_golden_vectors(path):
    z, hs, cams, prevs, di, W, H, frames = load_di_case(path)
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    ctx.counters(reset=True)
    res = []
    for f in range(frames):
        fr.render_di(scene, cams[f], prevs[f], di)   # G-buffer + DI pass, no indirect pass
        res.append({"resv": fr.download(G.BUF_DI_RESERVOIR), "temp": fr.download(G.BUF_DI_TEMP),
                    "out": fr.download(G.BUF_DIRECT_OUTPUT)})
    ctx.sync()
    check_di(z, res, ctx.counters(reset=True), frames)
    fr.close(); scene.close(); ctx.close()
