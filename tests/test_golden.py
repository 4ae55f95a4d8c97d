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
FILES = [p for p in ALL if not os.path.basename(p).startswith(("di_", "post_"))]
PNG_FILES = [p for p in ALL if os.path.basename(p).startswith("post_")]
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


def _png_pixels(path):
    """RGBA bytes of a PNG written by grisWritePNG (stored deflate blocks, filter 0 rows)."""
    import struct
    import zlib
    data = open(path, "rb").read()
    pos, idat, W, H = 8, b"", 0, 0
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            W, H = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    rows = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(H, W * 4 + 1)
    return rows[:, 1:].reshape(-1, 4), W, H


def _png_case(path):
    z = np.load(path)
    kind, grid, spheres, W, H, frames = [int(x) for x in z["meta"]]
    hs = G.HostScene(kind, seed=3, grid=grid, spheres=spheres)
    h = hashlib.sha256()
    for a in hs.arrays():
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(z["scene_sha256"])
    cams = [G.Camera.from_buffer_copy(bytes(c)) for c in z["cams"]]
    prevs = [G.Camera.from_buffer_copy(bytes(c)) for c in z["prevs"]]
    return (hs, cams, prevs, G.Settings.from_buffer_copy(bytes(z["settings"])),
            G.DISettings.from_buffer_copy(bytes(z["di_settings"])),
            G.PostSettings.from_buffer_copy(bytes(z["post_settings"])), W, H)


@pytest.mark.parametrize("path", PNG_FILES, ids=[os.path.basename(p)[:-4] for p in PNG_FILES])
def test_oracle_reproduces_golden_image(path):
    """Visual regression: the frame with both passes, presented, equals the committed image."""
    want, W0, H0 = _png_pixels(path[:-4] + ".png")
    hs, cams, prevs, st, di, post, W, H = _png_case(path)
    assert (W, H) == (W0, H0)
    ora = O.oracle()
    ora.set_scene(hs)
    ind = O.run_sequence(ora, cams, prevs, st, W, H, record=("out",))[-1]["out"]
    dirr = O.run_di_sequence(ora, ora, cams, prevs, di, W, H, record=("out",))[-1]["out"]
    _, rgba = O.post_process(W, H, dirr, ind, post)
    assert rgba.tobytes() == want.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("path", PNG_FILES, ids=[os.path.basename(p)[:-4] for p in PNG_FILES])
def test_gpu_reproduces_golden_image(path):
    import torch
    want, _, _ = _png_pixels(path[:-4] + ".png")
    hs, cams, prevs, st, di, post, W, H = _png_case(path)
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    for f in range(len(cams)):
        fr.render_di(scene, cams[f], prevs[f], di, st)
    dptr, _ = fr.device_ptr(G.BUF_DIRECT_OUTPUT)
    iptr, _ = fr.device_ptr(G.BUF_OUTPUT)
    dev = torch.zeros((W * H, 4), dtype=torch.uint8, device="cuda")
    ctx.post_process(G.PostBindings(W, H, dptr, iptr, 0, dev.data_ptr()), post)
    ctx.sync()
    assert dev.cpu().numpy().tobytes() == want.tobytes()
    fr.close(); scene.close(); ctx.close()
