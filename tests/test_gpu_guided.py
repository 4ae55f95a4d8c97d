"""Guided path sampling in a batch (grisBatchSetGuide): the guided estimator converges to the same
image as the unguided one (the guide only changes how suffix directions are drawn, with the
one-sample MIS pdf), the network trains on the rendered paths, and once trained it lowers the
error of a frame against the converged image on the glossy scene."""
import ctypes

import numpy as np
import pytest

import grisrt as G

pytestmark = pytest.mark.gpu


def _static_cams(hs, frames, W, H, seed):
    """One camera (the scene's first), a new seed per frame, no accumulation."""
    c0 = hs.camera(0, 60, W, H)
    cams, prevs = [], []
    for f in range(frames):
        c = c0.copy()
        c.seed = G.frame_seed(seed, f)
        ctypes.memmove(c.lastProjView, c0.projView, 64)
        c.frameIndex = G.CLEAR_FLAG if f == 0 else 0
        cams.append(c)
        prevs.append(c0.copy())
    return cams, prevs


def _converged(ctx, scene, cam, st, W, H, spp):
    import torch
    n = W * H
    dn = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    am = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    mv = torch.zeros((n, 2), dtype=torch.int16, device="cuda")
    gb = G.GBufferBindings(W, H, dn.data_ptr(), am.data_ptr(), mv.data_ptr())
    lib = G.load()
    ctx.check(lib.grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cam)), "grisPassGBuffer")
    s = torch.zeros(n * 3, dtype=torch.float64, device="cuda")
    q = torch.zeros(n * 3, dtype=torch.float64, device="cuda")
    for k in range(0, spp, 1024):
        scene.converged(cam, st, W, H, dn.data_ptr(), am.data_ptr(), s.data_ptr(), q.data_ptr(), spp_begin=k,
                        spp=min(1024, spp - k), estimator=G.ESTIMATOR_CANDIDATES)
    ctx.sync()
    mean = s.cpu().numpy().reshape(-1, 3) / spp
    var = np.maximum(q.cpu().numpy().reshape(-1, 3) / spp - mean ** 2, 0.0)
    return mean, var


def _render(ctx, scene, W, H, cams, prevs, st, guide=None):
    batch = G.Batch(ctx, [scene], [(W, H)])
    if guide is not None:
        batch.set_guide(guide)
    frames = []
    for c, p in zip(cams, prevs):
        batch.render([c], [p], [st])
        frames.append(batch.download(0, G.BUF_OUTPUT)[:, :3].astype(np.float64))
    ctx.sync()
    assert ctx.counters()[3] == 0
    batch.close()
    return np.stack(frames)


@pytest.mark.parametrize("tensor_cores", [False, True], ids=["mma_sync", "tcgen05"])
def test_guided_estimator_is_unbiased_and_trains_to_lower_error(tensor_cores):
    W, H, F = 48, 48, 384
    ctx = G.Context(0)
    ctx.set_path_form(G.PATH_WAVEFRONT)
    hs = G.HostScene(2, seed=1, grid=64, spheres=60)
    scene = G.Scene(ctx, hs)
    st = G.Settings.make(maxDepth=6, temporalReuse=False, spatialReuse=False)
    cams, prevs = _static_cams(hs, F, W, H, seed=21)
    ref, ref_var = _converged(ctx, scene, cams[0], st, W, H, 1 << 14)

    plain = _render(ctx, scene, W, H, cams, prevs, st)
    guide = G.Guide(ctx, G.GuideConfig.make(seed=5, samplesPerFrame=1 << 14, stepsPerFrame=2, learningRate=2e-3,
                                            tensorCores=tensor_cores))
    guided = _render(ctx, scene, W, H, cams, prevs, st, guide)
    trained = guide.get_params()
    assert np.all(np.isfinite(trained))
    assert np.abs(trained).sum() > 0

    def energy_test(frames, name):
        # the image sums of 16 independent chunks of frames against the converged image's sum
        chunks = frames.reshape(16, -1, W * H, 3).mean(axis=1).sum(axis=(1, 2))
        mean, se = chunks.mean(), chunks.std(ddof=1) / np.sqrt(len(chunks))
        se = np.sqrt(se ** 2 + ref_var.sum() / (1 << 14))
        z = (mean - ref.sum()) / se
        print("%s: image sum %.4f vs converged %.4f (z = %.2f)" % (name, mean, ref.sum(), z))
        return z

    assert abs(energy_test(plain, "plain")) < 4.0
    assert abs(energy_test(guided, "guided")) < 4.0

    def frame_error(frames):
        e = np.mean((frames - ref[None]) ** 2 / (ref[None] ** 2 + 1e-2), axis=2)
        return np.mean(e, axis=1)   # relMSE per frame

    ep, eg = frame_error(plain), frame_error(guided)
    late = slice(F // 2, F)
    print("relMSE per frame, second half: plain %.4f guided %.4f (median %.4f / %.4f)" % (
        ep[late].mean(), eg[late].mean(), np.median(ep[late]), np.median(eg[late])))
    assert np.median(eg[late]) < np.median(ep[late])
    guide.close()
    scene.close()
    ctx.close()
