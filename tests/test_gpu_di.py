"""ReSTIR DI on the GPU (grisPassDI / grisFrameRenderDI) against the oracle, bit for bit: the
candidate, temporal and spatial reservoirs, the direct output and the ray counts, for every shift
and sample type; the pass on caller buffers with a subset of its kernels; and the renderer's
frame with both the DI and the GRIS pass, whose GRIS buffers equal a frame without DI."""
import ctypes

import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

R, P, H = G.DI_SHIFT_RECONNECTION, G.DI_SHIFT_REPLAY, G.DI_SHIFT_HYBRID
L, B, BOTH = G.DI_SAMPLE_LIGHT, G.DI_SAMPLE_BSDF, G.DI_SAMPLE_BOTH

CASES = [
    ("box_reference_defaults", 0, 0, 0, 64, 48, 4, dict()),
    ("box_temporal_light", 0, 0, 0, 48, 40, 5, dict(temporalReuse=True)),
    ("box_replay_both", 0, 0, 0, 40, 32, 3, dict(shiftType=P, sampleType=BOTH, temporalReuse=True)),
    ("box_bsdf_reconnect", 0, 0, 0, 40, 32, 3, dict(sampleType=B, temporalReuse=True)),
    ("box_hybrid_no_merge", 0, 0, 0, 24, 24, 3, dict(shiftType=H, sampleType=BOTH, temporalReuse=True)),
    ("terrain_both", 1, 48, 60, 48, 40, 4, dict(sampleType=BOTH, temporalReuse=True)),
    ("terrain_replay_light", 1, 48, 60, 48, 40, 3, dict(shiftType=P, temporalReuse=True)),
    ("glossy_reconnect_both", 2, 48, 60, 48, 40, 3, dict(sampleType=BOTH, temporalReuse=True)),
    ("odd_size", 1, 32, 20, 37, 23, 3, dict(sampleType=BOTH, temporalReuse=True)),
]


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def gpu_di(ctx, hs, cams, prevs, di, W, H_, settings=None):
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H_)
    ctx.counters(reset=True)
    out = []
    for f in range(len(cams)):
        fr.render_di(scene, cams[f], prevs[f], di, settings)
        rec = {"resv": fr.download(G.BUF_DI_RESERVOIR), "temp": fr.download(G.BUF_DI_TEMP),
               "out": fr.download(G.BUF_DIRECT_OUTPUT)}
        if settings is not None:
            rec["gris_resv"] = fr.download(G.BUF_RESERVOIR)
            rec["gris_out"] = fr.download(G.BUF_OUTPUT)
        out.append(rec)
    ctx.sync()
    counters = ctx.counters(reset=True)
    fr.close()
    scene.close()
    return out, counters


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_di_matches_oracle(ctx, case):
    name, kind, grid, spheres, W, H_, frames, kw = case
    hs = G.HostScene(kind, seed=4, grid=grid, spheres=spheres)
    cams, prevs = G.sequence_cameras(hs, frames, W, H_, seed=17)
    di = G.DISettings.make(**kw)
    ora = O.oracle()
    ora.set_scene(hs)
    ora.read_counters(reset=True)
    want = O.run_di_sequence(ora, ora, cams, prevs, di, W, H_)
    cw = ora.read_counters(reset=True)
    got, cg = gpu_di(ctx, hs, cams, prevs, di, W, H_)
    for f in range(frames):
        for k in ("resv", "temp", "out"):
            assert got[f][k].tobytes() == want[f][k].tobytes(), "frame %d %s differs" % (f, k)
    assert list(cg[:3]) == list(cw[:3]) and cg[3] == 0


def test_gpu_di_pass_on_caller_buffers(ctx):
    """grisPassDI with torch buffers: bit 0 alone writes only This; then bits 1 and 2 give the
    full pass's result."""
    import torch
    hs = G.HostScene(0, seed=4)
    W, H_ = 40, 32
    cams, prevs = G.sequence_cameras(hs, 2, W, H_, seed=9)
    di = G.DISettings.make(sampleType=BOTH, temporalReuse=True)
    ora = O.oracle()
    ora.set_scene(hs)
    want = O.run_di_sequence(ora, ora, cams, prevs, di, W, H_)
    scene = G.Scene(ctx, hs)
    n = W * H_
    dev = "cuda"
    dn = [torch.zeros((n, 4), dtype=torch.float32, device=dev) for _ in range(2)]
    am = [torch.zeros((n, 2), dtype=torch.int32, device=dev) for _ in range(2)]
    mv = torch.zeros((n, 2), dtype=torch.int16, device=dev)
    resv = [torch.zeros((n, 16), dtype=torch.int32, device=dev) for _ in range(2)]
    temp = torch.zeros((n, 16), dtype=torch.int32, device=dev)
    out = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    lib = G.load()
    for f in range(2):
        j = f & 1
        gb = G.GBufferBindings(W, H_, dn[j].data_ptr(), am[j].data_ptr(), mv.data_ptr())
        ctx.check(lib.grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cams[f])), "grisPassGBuffer")
        b = G.DIBindings(W, H_, dn[j].data_ptr(), dn[j ^ 1].data_ptr(), am[j].data_ptr(), am[j ^ 1].data_ptr(),
                         mv.data_ptr(), resv[j].data_ptr(), resv[j ^ 1].data_ptr(), temp.data_ptr(), out.data_ptr())
        before_temp = temp.clone()
        ctx.pass_di(scene, b, cams[f], prevs[f], di, passes=1)
        ctx.sync()
        assert torch.equal(temp, before_temp)   # bit 0 leaves the temporary reservoirs alone
        ctx.pass_di(scene, b, cams[f], prevs[f], di, passes=6)
        ctx.sync()
        got = resv[j].cpu().numpy().view(G.DI_RESERVOIR).reshape(-1)
        assert got.tobytes() == want[f]["resv"].tobytes()
        assert temp.cpu().numpy().tobytes() == want[f]["temp"].tobytes()
        assert out.cpu().numpy().tobytes() == want[f]["out"].tobytes()
    # incomplete bindings are refused before any work
    bad = G.DIBindings(W, H_, dn[0].data_ptr(), 0, am[0].data_ptr(), 0, 0, resv[0].data_ptr(), 0, temp.data_ptr(), 0)
    with pytest.raises(G.GrisError):
        ctx.pass_di(scene, bad, cams[0], prevs[0], di, passes=7)
    scene.close()


def test_gpu_frame_with_direct_and_indirect(ctx):
    """grisFrameRenderDI with GRIS settings: the DI buffers equal the DI-only frame's and the GRIS
    buffers equal grisFrameRender's (the passes share only the G-buffer)."""
    hs = G.HostScene(1, seed=4, grid=40, spheres=40)
    W, H_ = 48, 40
    cams, prevs = G.sequence_cameras(hs, 3, W, H_, seed=7)
    di = G.DISettings.make(sampleType=BOTH, temporalReuse=True)
    st = G.Settings.make(maxDepth=5)
    both, _ = gpu_di(ctx, hs, cams, prevs, di, W, H_, settings=st)
    direct, _ = gpu_di(ctx, hs, cams, prevs, di, W, H_)
    scene = G.Scene(ctx, hs)
    fr = G.Frame(ctx, W, H_)
    for f in range(3):
        fr.render(scene, cams[f], prevs[f], st)
        assert both[f]["gris_resv"].tobytes() == fr.download(G.BUF_RESERVOIR).tobytes()
        assert both[f]["gris_out"].tobytes() == fr.download(G.BUF_OUTPUT).tobytes()
        for k in ("resv", "temp", "out"):
            assert both[f][k].tobytes() == direct[f][k].tobytes()
    fr.close()
    scene.close()


def test_gpu_di_full_hd_properties(ctx):
    """1920 x 1080, the C2-size terrain with both sample types and both reuse passes: finite
    output, M within the cap, every kept sample a light-instance hit, and the kernels' ray counts
    within their per-pixel bounds (candidates <= 2, temporal <= 2, spatial <= 11 per pixel)."""
    hs = G.HostScene(1, seed=1, grid=256, spheres=400)
    W, H_ = 1920, 1080
    cams, prevs = G.sequence_cameras(hs, 3, W, H_, seed=3)
    di = G.DISettings.make(sampleType=BOTH, temporalReuse=True)
    got, c = gpu_di(ctx, hs, cams, prevs, di, W, H_)
    r = got[-1]["resv"]
    assert np.isfinite(got[-1]["out"]).all()
    assert r["sampleCount"].max() <= 40
    valid = r["instanceIdx"] != G.INVALID_HIT
    assert valid.any() and np.all(r["instanceIdx"][valid] == 0)
    px = W * H_ * 3
    assert c[0] + c[1] <= px * (2 + 2 + 11) and c[3] == 0
