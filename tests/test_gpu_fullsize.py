"""Full-size checks at the benchmark configurations (C1: 256x256 box, 8 frames; C2: 1920x1080,
1.16M triangles, depth 8; C2 glossy variant): the CUDA path against the oracle (binary-BVH
traversal, equal to brute force ray by ray) bit for bit, plus size-independent properties
(determinism across runs, reservoir invariants)."""
import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def run_gpu(hs, cams, prevs, st, W, H, keep=("resv", "temp", "out"), refill=0):
    ctx = G.Context(0)
    ctx.set_wave_refill(refill)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    ctx.counters(reset=True)
    res = []
    which = {"resv": G.BUF_RESERVOIR, "temp": G.BUF_TEMP, "out": G.BUF_OUTPUT, "dn": G.BUF_DEPTH_NORMAL,
             "am": G.BUF_ALBEDO_MATID, "mv": G.BUF_MOTION}
    for f in range(len(cams)):
        fr.render(scene, cams[f], prevs[f], st)
        res.append({k: fr.download(which[k]) for k in keep})
    ctx.sync()
    cnt = ctx.counters(reset=True)
    fr.close(); scene.close(); ctx.close()
    return res, cnt


def run_oracle(hs, cams, prevs, st, W, H, keep=("resv", "temp", "out")):
    ora = O.oracle()
    ora.set_scene(hs)
    ora.set_traversal(True)
    ora.read_counters(reset=True)
    res = O.run_sequence(ora, cams, prevs, st, W, H, record=keep)
    return res, ora.read_counters(reset=True)


def assert_same(got, want, frames, keys):
    for f in range(frames):
        for k in keys:
            g, w = got[f][k], want[f][k]
            if g.tobytes() != w.tobytes():
                gv = g.view(np.uint32).reshape(len(g), -1)
                wv = w.view(np.uint32).reshape(len(w), -1)
                bad = np.nonzero((gv != wv).any(1))[0]
                pytest.fail("frame %d %s: %d pixels differ, first %s" % (f, k, len(bad), bad[:8]))


def check_invariants(resv, cap):
    valid = resv["instanceIdx"] != G.INVALID_HIT
    assert np.all(resv["sampleCount"][valid] <= cap)
    w = resv["resampleWeight"]
    assert np.all(np.isfinite(w[valid])) and np.all(w[valid] >= 0)
    flags = resv["flags"][valid]
    assert np.all((flags >> 16) & 0xff <= 2)               # rc vertex type
    assert np.all((flags & 0xff) <= ((flags >> 8) & 0xff))  # rc vertex within the path


def test_c1_box_256_8_frames_full_parity():
    W = H = 256
    hs = G.HostScene(0, seed=1)
    cams, prevs = G.sequence_cameras(hs, 8, W, H, seed=1)
    st = G.Settings.make(maxDepth=3, spatialRadius=30.0, cap=20)
    got, gc = run_gpu(hs, cams, prevs, st, W, H, keep=("resv", "temp", "out", "dn", "am", "mv"))
    want, oc = run_oracle(hs, cams, prevs, st, W, H, keep=("resv", "temp", "out", "dn", "am", "mv"))
    assert_same(got, want, 8, ("dn", "am", "mv", "resv", "temp", "out"))
    assert gc[:3] == oc[:3]
    for f in range(8):
        check_invariants(got[f]["resv"], 20)


@pytest.mark.parametrize("kind", [1, 2], ids=["c2_plain", "c4_glossy"])
def test_c2_1080p_full_parity(kind):
    """Both wavefront traversals (one lane per ray over the level's queue; the resident walks that
    refill lanes, with the one-ray-per-warp walk of sparse levels) against the oracle on the full
    frame."""
    W, H = 1920, 1080
    hs = G.HostScene(kind, seed=1, grid=512, spheres=2000)
    assert hs.triangle_count() > 1_100_000
    cams, prevs = G.sequence_cameras(hs, 3, W, H, seed=1, orbit_frames=60)
    st = G.Settings.make(maxDepth=8, spatialRadius=20.0, cap=20)
    want, oc = run_oracle(hs, cams, prevs, st, W, H)
    for refill in (0, 1):
        got, gc = run_gpu(hs, cams, prevs, st, W, H, refill=refill)
        assert_same(got, want, 3, ("resv", "temp", "out"))
        assert gc[:3] == oc[:3], refill
        assert gc[3] == 0, refill
        for f in range(3):
            check_invariants(got[f]["resv"], 20)


def test_c2_1080p_is_deterministic():
    W, H = 1920, 1080
    hs = G.HostScene(1, seed=2, grid=512, spheres=2000)
    cams, prevs = G.sequence_cameras(hs, 4, W, H, seed=5, orbit_frames=60)
    st = G.Settings.make(maxDepth=8)
    a, ca = run_gpu(hs, cams, prevs, st, W, H)
    b, cb = run_gpu(hs, cams, prevs, st, W, H)
    assert_same(a, b, 4, ("resv", "temp", "out"))
    assert ca == cb
    out = a[-1]["out"]
    assert np.all(np.isfinite(out)) and np.all(out[:, :3] >= 0) and np.all(out[:, :3] <= 1e4)
