"""Pairwise MIS weights for the reuse passes (GrisSettings.misWeights = 1, an extension): with
temporal + spatial reuse and frames accumulated under a static camera on the glossy scene, the
reference's merge drifts away from the converged image (its image energy rises frame after
frame), while the pairwise generalised balance heuristic keeps the accumulated image at the
converged image's energy and lowers its error."""
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
        energy.append(img.sum() / ref.sum())
        e = np.mean((img - ref) ** 2 / (ref * ref + 1e-2), axis=1)
        med.append(float(np.median(e[fg])))
    ctx.sync()
    assert ctx.counters()[3] == 0
    batch.close()
    return np.array(energy), np.array(med)


def test_pairwise_weights_remove_the_energy_drift():
    W, H, F = 640, 360, 24
    ctx = G.Context(0)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    hs = G.HostScene(2, seed=1, grid=256, spheres=600)
    scene = G.Scene(ctx, hs)
    c0, cams, prevs = _static_accumulating_cams(hs, F, W, H, seed=7)
    ref_st = G.Settings.make(maxDepth=10)
    ref = _converged(ctx, scene, c0, ref_st, W, H, 1024)
    e_ref, m_ref = _accumulate(ctx, scene, cams, prevs, G.Settings.make(maxDepth=10), W, H, ref)
    e_pw, m_pw = _accumulate(ctx, scene, cams, prevs, G.Settings.make(maxDepth=10, misWeights=1), W, H, ref)
    print("energy, reference merge:", np.round(e_ref[::4], 3), "pairwise:", np.round(e_pw[::4], 3))
    print("median error, reference merge:", np.round(m_ref[::4], 4), "pairwise:", np.round(m_pw[::4], 4))
    # the accumulated pairwise image stays at the converged image's energy
    assert abs(e_pw[-1] - 1.0) < 0.05
    assert abs(e_pw[-1] - 1.0) < abs(e_ref[-1] - 1.0)
    assert m_pw[-1] < m_ref[-1]
    scene.close()
    ctx.close()


def test_pairwise_weights_on_the_lambertian_box():
    """Where every shift succeeds both ways, both merges converge; pairwise stays unbiased."""
    W, H, F = 128, 128, 32
    ctx = G.Context(0)
    hs = G.HostScene(0, seed=1)
    scene = G.Scene(ctx, hs)
    c0, cams, prevs = _static_accumulating_cams(hs, F, W, H, seed=3)
    st = G.Settings.make(maxDepth=4, spatialRadius=30.0, misWeights=1)
    ref = _converged(ctx, scene, c0, G.Settings.make(maxDepth=4), W, H, 4096)
    e_pw, m_pw = _accumulate(ctx, scene, cams, prevs, st, W, H, ref)
    print("box energy, pairwise:", np.round(e_pw[::4], 4), "median error", np.round(m_pw[::4], 5))
    assert abs(e_pw[-1] - 1.0) < 0.02
    assert m_pw[-1] < 0.25 * m_pw[0]
    scene.close()
    ctx.close()


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
