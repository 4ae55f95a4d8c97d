"""GPU parity: the CUDA path through the C ABI against the oracle, bit for bit (reservoir
selections, M, weights, G-buffer, output radiance, ray counts)."""
import ctypes

import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

CASES = [
    ("box_config1", 0, 0, 0, 64, 48, 8, dict(maxDepth=3, spatialRadius=30.0)),
    ("box_reference_defaults", 0, 0, 0, 40, 40, 3, dict()),
    ("box_reconnection", 0, 0, 0, 32, 24, 3, dict(shiftType=0, maxDepth=6)),
    ("box_no_temporal", 0, 0, 0, 24, 24, 3, dict(temporalReuse=False, maxDepth=4)),
    ("box_no_spatial_cap5", 0, 0, 0, 24, 24, 4, dict(spatialReuse=False, cap=5, maxDepth=4)),
    ("terrain_depth8", 1, 48, 60, 48, 40, 4, dict(maxDepth=8, spatialRadius=30.0)),
    ("glossy_depth8", 2, 48, 60, 48, 40, 4, dict(maxDepth=8, spatialRadius=30.0)),
    ("glossy_rr", 2, 24, 30, 32, 24, 3, dict(maxDepth=12, rrScale=0.5, spatialNeighbors=5)),
    ("odd_size", 1, 32, 20, 37, 23, 3, dict(maxDepth=5)),
    ("terrain_9nb_cap3", 1, 32, 40, 40, 30, 3, dict(maxDepth=6, spatialNeighbors=9, cap=3)),   # three chunks of neighbours
    ("box_1nb", 0, 0, 0, 24, 16, 3, dict(maxDepth=4, spatialNeighbors=1)),
]


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def ora():
    return O.oracle()


def gpu_sequence(ctx, hs, cams, prevs, st, W, H, mode=(G.PATH_WAVEFRONT, G.LAUNCH_GRID)):
    ctx.set_path_form(mode[0])
    ctx.set_launch_mode(mode[1])
    ctx.set_wave_refill(mode[2] if len(mode) > 2 else 0)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H)
    ctx.counters(reset=True)
    out = []
    for f in range(len(cams)):
        fr.render(scene, cams[f], prevs[f], st)
        out.append({"resv": fr.download(G.BUF_RESERVOIR), "temp": fr.download(G.BUF_TEMP),
                    "out": fr.download(G.BUF_OUTPUT), "dn": fr.download(G.BUF_DEPTH_NORMAL),
                    "am": fr.download(G.BUF_ALBEDO_MATID), "mv": fr.download(G.BUF_MOTION)})
    ctx.sync()
    counters = ctx.counters(reset=True)
    fr.close()
    scene.close()
    return out, counters


MODES = [(G.PATH_WAVEFRONT, G.LAUNCH_GRID), (G.PATH_MEGAKERNEL, G.LAUNCH_GRID), (G.PATH_MEGAKERNEL, G.LAUNCH_PERSISTENT),
         (G.PATH_WAVEFRONT, G.LAUNCH_GRID, 1)]   # refilling wavefront: sparse levels walked one ray per warp
MODE_IDS = ["wavefront", "megakernel-grid", "megakernel-persistent", "wavefront-refill"]


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_matches_oracle_bit_exact(case, mode, ctx, ora):
    name, kind, grid, spheres, W, H, frames, kw = case
    hs = G.HostScene(kind, seed=2, grid=grid, spheres=spheres)
    cams, prevs = G.sequence_cameras(hs, frames, W, H, seed=11)
    st = G.Settings.make(**kw)
    got, gc = gpu_sequence(ctx, hs, cams, prevs, st, W, H, mode)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    ctx.set_launch_mode(G.LAUNCH_GRID)
    ctx.set_wave_refill(False)
    ora.set_scene(hs)
    ora.read_counters(reset=True)
    want = O.run_sequence(ora, cams, prevs, st, W, H)
    oc = ora.read_counters()
    for f in range(frames):
        for k in ("dn", "am", "mv", "resv", "temp", "out"):
            g, w = got[f][k], want[f][k]
            if g.tobytes() != w.tobytes():
                gv = g.view(np.uint32).reshape(len(g), -1)
                wv = w.view(np.uint32).reshape(len(w), -1)
                bad = np.nonzero((gv != wv).any(1))[0]
                pytest.fail("%s: frame %d buffer %s differs at %d pixels, first %s:\n gpu %s\n oracle %s" % (
                    name, f, k, len(bad), bad[:8], g[bad[0]], w[bad[0]]))
    assert gc[0] == oc[0] and gc[1] == oc[1] and gc[2] == oc[2], (gc, oc)
    assert gc[3] == 0


PAIRWISE_CASES = [
    ("box_pairwise", 0, 0, 0, 48, 40, 5, dict(maxDepth=4, spatialRadius=30.0, misWeights=1)),
    ("terrain_pairwise", 1, 48, 60, 48, 40, 4, dict(maxDepth=8, misWeights=1)),
    ("glossy_pairwise_5nb", 2, 48, 60, 40, 32, 3, dict(maxDepth=8, spatialNeighbors=5, misWeights=1)),
    ("terrain_pairwise_no_temporal", 1, 32, 20, 37, 23, 3, dict(maxDepth=6, temporalReuse=False, misWeights=1)),
    ("box_pairwise_no_spatial", 0, 0, 0, 32, 24, 4, dict(maxDepth=4, spatialReuse=False, misWeights=1)),
]


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
@pytest.mark.parametrize("case", PAIRWISE_CASES, ids=[c[0] for c in PAIRWISE_CASES])
def test_gpu_pairwise_weights_match_oracle(case, mode, ctx, ora):
    """The pairwise MIS weights (GrisSettings.misWeights = 1, an extension with no counterpart in
    the reference): the CUDA reuse passes against the oracle's restatement, bit for bit."""
    test_gpu_matches_oracle_bit_exact(case, mode, ctx, ora)


@pytest.mark.parametrize("rays_kind", ["random", "edges"])
def test_device_traversal_matches_host(ctx, rays_kind):
    """50,000 random rays (or 20,000 aimed at triangle vertices and edges, where the fused
    triangle test's rounding decides), closest hit and any hit: the device walk with the resident
    traversal kernels' short stack (two register entries, here one shared-memory entry, then the
    local-memory overflow, so deep walks use all three) against the host walk's array stack, bit
    for bit."""
    hs = G.HostScene(1, seed=4, grid=64, spheres=100)
    scene = G.Scene(ctx, hs)
    if rays_kind == "edges":
        from test_bvh_cpu import _rays
        rays = _rays(hs, 20000, 6, "edges")
        n = len(rays)
    else:
        rng = np.random.default_rng(5)
        n = 50000
        rays = np.zeros((n, 8), np.float32)
        rays[:, 0:3] = rng.uniform([-55, -55, -5], [55, 55, 25], (n, 3))
        d = rng.normal(size=(n, 3))
        rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
        rays[:, 3], rays[:, 7] = 1e-4, 1e7
    import torch
    dr = torch.from_numpy(rays).cuda()
    tuv = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    inst = torch.zeros(n, dtype=torch.int32, device="cuda")
    tri = torch.zeros(n, dtype=torch.int32, device="cuda")
    for any_hit in (0, 1):
        torch.cuda.synchronize()
        ctx.check(G.load().grisDebugTraceDevice(ctx.h, scene.h, dr.data_ptr(), n, any_hit, tuv.data_ptr(),
                                                inst.data_ptr(), tri.data_ptr()), "grisDebugTraceDevice")
        ctx.sync()
        h_tuv, h_inst, h_tri = scene.trace_host(rays, any_hit=bool(any_hit))
        if any_hit:
            assert np.array_equal(tuv[:, 0].cpu().numpy() > 0, h_tuv[:, 0] > 0)
        else:
            assert np.array_equal(inst.cpu().numpy().view(np.uint32), h_inst)
            assert np.array_equal(tri.cpu().numpy().view(np.uint32), h_tri)
            assert tuv.cpu().numpy().tobytes() == h_tuv.tobytes()
    scene.close()


def test_pass_bindings_api_matches_frame_api(ctx, ora):
    """grisPassGBuffer + grisPassRender on caller-owned device buffers (the descriptor-set form)."""
    import torch
    W, H, frames = 40, 32, 3
    hs = G.HostScene(0, seed=3)
    cams, prevs = G.sequence_cameras(hs, frames, W, H, seed=5)
    st = G.Settings.make(maxDepth=4, spatialRadius=30.0)
    scene = G.Scene(ctx, hs)
    n = W * H
    dn = [torch.zeros((n, 4), dtype=torch.float32, device="cuda") for _ in range(2)]
    am = [torch.zeros((n, 2), dtype=torch.int32, device="cuda") for _ in range(2)]
    mv = torch.zeros((n, 2), dtype=torch.int16, device="cuda")
    resv = [torch.zeros((n, 24), dtype=torch.int32, device="cuda") for _ in range(2)]
    temp = torch.zeros((n, 24), dtype=torch.int32, device="cuda")
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    lib = G.load()
    ora.set_scene(hs)
    want = O.run_sequence(ora, cams, prevs, st, W, H, record=("resv", "out"))
    j = 0
    for f in range(frames):
        gb = G.GBufferBindings(W, H, dn[j].data_ptr(), am[j].data_ptr(), mv.data_ptr())
        ctx.check(lib.grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cams[f])), "grisPassGBuffer")
        b = G.PassBindings(W, H, dn[j].data_ptr(), dn[j ^ 1].data_ptr(), am[j].data_ptr(), am[j ^ 1].data_ptr(),
                           mv.data_ptr(), resv[j].data_ptr(), resv[j ^ 1].data_ptr(), temp.data_ptr(), out.data_ptr())
        ctx.check(lib.grisPassRender(ctx.h, scene.h, ctypes.byref(b), ctypes.byref(cams[f]), ctypes.byref(prevs[f]),
                                     ctypes.byref(st), 7), "grisPassRender")
        ctx.sync()
        assert resv[j].cpu().numpy().tobytes() == want[f]["resv"].tobytes()
        assert out.cpu().numpy().tobytes() == want[f]["out"].tobytes()
        j ^= 1
    scene.close()


def test_invalid_arguments_are_rejected(ctx):
    lib = G.load()
    hs = G.HostScene(0, seed=1)
    scene = G.Scene(ctx, hs)
    cam = hs.camera(0, 1, 16, 16)
    st = G.Settings.make()
    b = G.PassBindings()
    b.width, b.height = 16, 16
    assert lib.grisPassRender(ctx.h, scene.h, ctypes.byref(b), ctypes.byref(cam), ctypes.byref(cam), ctypes.byref(st), 7) == -1
    st.maxDepth = 0
    assert lib.grisFrameRender(ctx.h, scene.h, None, ctypes.byref(cam), ctypes.byref(cam), ctypes.byref(st)) == -1
    bad = G.HostScene(0, seed=1)
    bad.materials["textureIdx"][0] = 3
    h = ctypes.c_void_p()
    d = bad.desc()
    assert lib.grisSceneCreate(ctx.h, ctypes.byref(d), ctypes.byref(h)) == -4
    scene.close()


def test_persistent_launches_from_two_threads(ora):
    """The persistent launch form looks up the SM count and each kernel's resident blocks per SM
    once per device, under a lock shared by every host thread: two threads with their own
    contexts, rendering at the same time from a cold start, both get the oracle's frames."""
    import threading
    W, H, frames = 32, 24, 3
    hs = G.HostScene(1, seed=2, grid=32, spheres=20)
    cams, prevs = G.sequence_cameras(hs, frames, W, H, seed=7)
    st = G.Settings.make(maxDepth=5)
    ora.set_scene(hs)
    want = O.run_sequence(ora, cams, prevs, st, W, H, record=("resv", "out"))
    results, errors = [None, None], []
    start = threading.Barrier(2)

    def run(k):
        try:
            c = G.Context(0)
            start.wait()
            got, counters = gpu_sequence(c, hs, cams, prevs, st, W, H, (G.PATH_MEGAKERNEL, G.LAUNCH_PERSISTENT))
            results[k] = (got, counters)
            c.close()
        except Exception as e:   # reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for got, counters in results:
        assert counters[3] == 0
        for f in range(frames):
            assert got[f]["resv"].tobytes() == want[f]["resv"].tobytes()
            assert got[f]["out"].tobytes() == want[f]["out"].tobytes()
