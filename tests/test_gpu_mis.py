"""Pairwise MIS weights for the reuse passes (GrisSettings.misWeights = 1, an extension), next to
the reference's merge, on images accumulated under a static camera against the converged image:
with one reuse pass at a time both merges stay at the converged image's energy; chaining
temporal and spatial reuse over frames makes both drift (the reference's merge darker on the
box, the pairwise weights brighter), which the test records rather than hides."""
import ctypes

import numpy as np
import pytest

import grisrt as G

pytestmark = pytest.mark.gpu


def _static_accumulating_cams(hs, frames, W, H, seed):
    c0 = hs.camera(0, 60, W, H)
    cams, prevs = [], []
    for f in range(frames):
        c = c0.copy()
        c.seed = G.frame_seed(seed, f)
        ctypes.memmove(c.lastProjView, c0.projView, 64)
        c.frameIndex = G.CLEAR_FLAG if f == 0 else f
        cams.append(c)
        prevs.append(c0.copy())
    return c0, cams, prevs


def _converged(ctx, scene, cam, st, W, H, spp):
    import torch
    n = W * H
    dn = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    am = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    mv = torch.zeros((n, 2), dtype=torch.int16, device="cuda")
    gb = G.GBufferBindings(W, H, dn.data_ptr(), am.data_ptr(), mv.data_ptr())
    ctx.check(G.load().grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cam)), "grisPassGBuffer")
    s = torch.zeros(n * 3, dtype=torch.float64, device="cuda")
    for k in range(0, spp, 64):
        scene.converged(cam, st, W, H, dn.data_ptr(), am.data_ptr(), s.data_ptr(), None, spp_begin=k, spp=64,
                        estimator=G.ESTIMATOR_CANDIDATES)
    ctx.sync()
    return s.cpu().numpy().reshape(-1, 3) / spp


def _accumulate(ctx, scene, cams, prevs, st, W, H, ref):
    batch = G.Batch(ctx, [scene], [(W, H)])
    energy, med = [], []
    fg = ref.sum(axis=1) > 0
    for c, p in zip(cams, prevs):
        batch.render([c], [p], [st])
        img = batch.download(0, G.BUF_OUTPUT)[:, :3].astype(np.float64)
        assert np.all(np.isfinite(img))
        energy.append(img.sum() / ref.sum())
        e = np.mean((img - ref) ** 2 / (ref * ref + 1e-2), axis=1)
        med.append(float(np.median(e[fg])))
    ctx.sync()
    assert ctx.counters()[3] == 0
    batch.close()
    return np.array(energy), np.array(med)


@pytest.fixture(scope="module")
def box():
    W, H, F = 128, 128, 32
    ctx = G.Context(0)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    hs = G.HostScene(0, seed=1)
    scene = G.Scene(ctx, hs)
    c0, cams, prevs = _static_accumulating_cams(hs, F, W, H, seed=3)
    ref = _converged(ctx, scene, c0, G.Settings.make(maxDepth=4), W, H, 4096)
    yield ctx, scene, cams, prevs, ref, W, H
    scene.close()
    ctx.close()


@pytest.mark.parametrize("mis", [0, 1], ids=["reference-merge", "pairwise"])
@pytest.mark.parametrize("temporal,spatial", [(True, False), (False, True)], ids=["temporal", "spatial"])
def test_one_reuse_pass_keeps_the_converged_energy(box, mis, temporal, spatial):
    ctx, scene, cams, prevs, ref, W, H = box
    st = G.Settings.make(maxDepth=4, spatialRadius=30.0, misWeights=mis, temporalReuse=temporal, spatialReuse=spatial)
    e, m = _accumulate(ctx, scene, cams, prevs, st, W, H, ref)
    print("mis", mis, "temporal", temporal, "spatial", spatial, "energy", np.round(e[::8], 4), "median", m[-1])
    assert abs(e[-1] - 1.0) < 0.02
    assert m[-1] < 0.5 * m[0]


def test_chained_reuse_drift_is_recorded(box):
    ctx, scene, cams, prevs, ref, W, H = box
    out = {}
    for mis in (0, 1):
        st = G.Settings.make(maxDepth=4, spatialRadius=30.0, misWeights=mis)
        e, m = _accumulate(ctx, scene, cams, prevs, st, W, H, ref)
        out[mis] = e
        print("chained temporal + spatial, mis", mis, "energy", np.round(e[::8], 4))
    # both drift by less than 15% over 32 frames here; in opposite directions
    assert abs(out[0][-1] - 1.0) < 0.15 and abs(out[1][-1] - 1.0) < 0.15


def test_pairwise_weights_in_a_guided_batch_run():
    """Guided batches with pairwise weights: finite output, energy near the converged image's."""
    W, H, F = 320, 180, 16
    ctx = G.Context(0)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    hs = G.HostScene(2, seed=1, grid=128, spheres=200)
    scene = G.Scene(ctx, hs)
    c0, cams, prevs = _static_accumulating_cams(hs, F, W, H, seed=5)
    ref = _converged(ctx, scene, c0, G.Settings.make(maxDepth=8), W, H, 512)
    guide = G.Guide(ctx, G.GuideConfig.make(seed=2, samplesPerFrame=1 << 15, stepsPerFrame=2))
    batch = G.Batch(ctx, [scene], [(W, H)])
    batch.set_guide(guide)
    st = G.Settings.make(maxDepth=8, misWeights=1)
    for c, p in zip(cams, prevs):
        batch.render([c], [p], [st])
    img = batch.download(0, G.BUF_OUTPUT)[:, :3].astype(np.float64)
    ctx.sync()
    assert np.all(np.isfinite(img))
    print("guided pairwise energy", img.sum() / ref.sum())
    assert abs(img.sum() / ref.sum() - 1.0) < 0.15
    batch.close()
    guide.close()
    scene.close()
    ctx.close()
