"""The converged image and its relMSE.

CPU: the FP64 oracle (oracle/converged_fp64.cpp) — its two estimators coincide where every
vertex is reconnectible, its sample ranges add up, and gi_naive's literal NEE weight of 1 counts
the light reached by both strategies twice.
GPU: grisConvergedAccumulate (FP32 paths, FP64 sums) agrees with the FP64 oracle within the
statistical error of both (a chi-square test over pixels); grisRelMSE equals the FP64 formula;
ReSTIR PT's frames are closer to the converged image than the canonical samples alone.
"""
import numpy as np
import pytest

import grisrt as G
from oracle import pyoracle as O


def _gbuffer_cpu(hs, cams, prevs, st, W, H):
    ora = O.oracle()
    ora.set_scene(hs)
    r = O.run_sequence(ora, cams[:1], prevs[:1], st, W, H, record=("dn", "am"))[0]
    return r["dn"], r["am"]


def test_fp64_estimators_agree_on_lambertian_box():
    hs = G.HostScene(0, seed=2)
    W, H = 24, 20
    cams, prevs = G.sequence_cameras(hs, 1, W, H, seed=5)
    st = G.Settings.make(maxDepth=4)
    dn, am = _gbuffer_cpu(hs, cams, prevs, st, W, H)
    f = O.ConvergedFP64()
    assert f.set_scene(hs) == 26
    m0, v0 = f.render(cams[0], st, W, H, dn, am, spp=256, estimator=0)
    m1, v1 = f.render(cams[0], st, W, H, dn, am, spp=256, estimator=1)
    # every vertex of the box is reconnectible: each path's candidates are all its contributions
    # (summed in another order)
    assert np.allclose(m0, m1, rtol=1e-12, atol=0.0)
    assert m0.max() > 0.0
    # gi_naive.glsl's NEE weight 1 adds the MIS-weighted light hits on top of full NEE
    m2, _ = f.render(cams[0], st, W, H, dn, am, spp=256, estimator=2)
    assert m2.sum() > m1.sum()


def test_fp64_sample_ranges_add_up():
    hs = G.HostScene(0, seed=3)
    W, H = 8, 8
    cams, prevs = G.sequence_cameras(hs, 1, W, H, seed=1)
    st = G.Settings.make(maxDepth=3)
    dn, am = _gbuffer_cpu(hs, cams, prevs, st, W, H)
    f = O.ConvergedFP64()
    f.set_scene(hs)
    a, _ = f.render(cams[0], st, W, H, dn, am, spp=32, spp_begin=0)
    b, _ = f.render(cams[0], st, W, H, dn, am, spp=32, spp_begin=32)
    c, _ = f.render(cams[0], st, W, H, dn, am, spp=64, spp_begin=0)
    assert np.allclose((a + b) / 2, c, rtol=1e-12, atol=1e-15)
    d, _ = f.render(cams[0], st, W, H, dn, am, spp=32, spp_begin=0, rect=(2, 3, 6, 7))
    full = a.reshape(H, W, 3)[3:7, 2:6].reshape(-1, 3)
    assert np.array_equal(d, full)


def _device_gbuffer(ctx, scene, cam, W, H):
    import ctypes
    import torch
    lib = G.load()
    n = W * H
    dn = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    am = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    mv = torch.zeros((n, 2), dtype=torch.int16, device="cuda")
    gb = G.GBufferBindings(W, H, dn.data_ptr(), am.data_ptr(), mv.data_ptr())
    ctx.check(lib.grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cam)), "grisPassGBuffer")
    ctx.sync()
    return dn, am


def _gpu_converged(ctx, scene, cam, st, W, H, spp, estimator, chunks=1):
    import torch
    dn, am = _device_gbuffer(ctx, scene, cam, W, H)
    s = torch.zeros(W * H * 3, dtype=torch.float64, device="cuda")
    q = torch.zeros(W * H * 3, dtype=torch.float64, device="cuda")
    per = spp // chunks
    for k in range(chunks):
        scene.converged(cam, st, W, H, dn.data_ptr(), am.data_ptr(), s.data_ptr(), q.data_ptr(), spp_begin=k * per,
                        spp=per, estimator=estimator)
    ctx.sync()
    assert ctx.counters()[3] == 0
    return s, q, dn, am


def _z2(m_a, v_a, n_a, m_b, v_b, n_b):
    se2 = v_a / n_a + v_b / n_b
    ok = se2 > 0
    z = (m_a[ok] - m_b[ok]) / np.sqrt(se2[ok])
    return z


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["box", "glossy"])
@pytest.mark.parametrize("estimator", [G.ESTIMATOR_CANDIDATES, G.ESTIMATOR_INDIRECT], ids=["candidates", "indirect"])
def test_gpu_converged_matches_fp64_oracle(case, estimator):
    if case == "box":
        hs, W, H, st = G.HostScene(0, seed=2), 32, 32, G.Settings.make(maxDepth=3)
        spp_gpu, spp_cpu = 1 << 16, 4096
    else:
        hs, W, H, st = G.HostScene(2, seed=1, grid=48, spheres=40), 24, 24, G.Settings.make(maxDepth=6)
        spp_gpu, spp_cpu = 1 << 16, 2048
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    cams, _ = G.sequence_cameras(hs, 1, W, H, seed=5)
    s, q, dn, am = _gpu_converged(ctx, scene, cams[0], st, W, H, spp_gpu, estimator, chunks=2)
    m_gpu = s.cpu().numpy().reshape(-1, 3) / spp_gpu
    v_gpu = np.maximum(q.cpu().numpy().reshape(-1, 3) / spp_gpu - m_gpu ** 2, 0.0)
    f = O.ConvergedFP64()
    f.set_scene(hs)
    m_cpu, v_cpu = f.render(cams[0], st, W, H, dn.cpu().numpy(), am.cpu().numpy().view(np.uint32), spp=spp_cpu,
                            seed=11, estimator=estimator)
    z = _z2(m_cpu, v_cpu, spp_cpu, m_gpu, v_gpu, spp_gpu)
    assert len(z) > 0.5 * W * H
    chi = float(np.mean(z * z))
    # both are unbiased estimates of one expectation: z^2 averages ~1 (heavy-tailed glossy paths
    # make the sample variance noisy, hence the wider band there)
    lo, hi = (0.8, 1.25) if case == "box" else (0.6, 1.6)
    assert lo < chi < hi, chi
    assert np.mean(np.abs(z) > 4.0) < 0.005
    # the images agree in total energy to within the error of the CPU mean
    tot_err = np.sqrt(v_cpu.sum() / spp_cpu)
    assert abs(m_cpu.sum() - m_gpu.sum()) < 5.0 * tot_err
    scene.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_relmse_reduction_equals_fp64_formula():
    import torch
    ctx = G.Context(0)
    rng = np.random.default_rng(4)
    n = 100_003
    img = rng.random((n, 4)).astype(np.float32) * 3.0
    ref = rng.random((n, 3)) * 2.0
    ref[::7] = 0.0
    ti = torch.from_numpy(img).cuda()
    tr = torch.from_numpy((ref * 16.0).reshape(-1)).cuda()
    got = ctx.relmse(ti.data_ptr(), tr.data_ptr(), 1.0 / 16.0, n, eps=1e-2)
    d = img[:, :3].astype(np.float64) - ref
    want_rel = np.mean(d * d / (ref * ref + 1e-2))
    want_mse = np.mean(d * d)
    assert abs(got[0] - want_rel) <= 1e-12 * want_rel
    assert abs(got[1] - want_mse) <= 1e-12 * want_mse
    assert ctx.relmse(ti.data_ptr(), tr.data_ptr(), 1.0 / 16.0, n, eps=1e-2) == got   # fixed summation order
    ctx.close()


@pytest.mark.gpu
def test_restir_frames_approach_the_converged_image():
    """Error against the converged image: frames with temporal + spatial reuse beat the
    canonical sample alone, and accumulating frames (static camera) keeps lowering it. The
    per-pixel median of the squared relative error is the measure; the relMSE (its mean) is
    printed beside it: reused samples with large weights (fireflies) persist for a few frames
    under the 1/M-style merge of the reference, so the mean is not monotone."""
    import torch
    hs, W, H = G.HostScene(0, seed=1), 64, 64
    ctx = G.Context(0)
    scene = G.Scene(ctx, hs)
    st = G.Settings.make(maxDepth=3, spatialRadius=30.0)
    cams, prevs = G.sequence_cameras(hs, 16, W, H, seed=9)
    s, _, _, _ = _gpu_converged(ctx, scene, cams[0], st, W, H, 1 << 16, G.ESTIMATOR_CANDIDATES)
    scale = 1.0 / (1 << 16)
    ref = s.cpu().numpy().reshape(-1, 3) * scale
    fg = ref.sum(axis=1) > 0

    def run(settings, accumulate, frames):
        fr = G.Frame(ctx, W, H)
        cs, ps = G.sequence_cameras(hs, frames, W, H, seed=9, accumulate=accumulate)
        rel, med = [], []
        for f in range(frames):
            fr.render(scene, cs[f], ps[f], settings)
            ptr, _ = fr.device_ptr(G.BUF_OUTPUT)
            r = ctx.relmse(ptr, s.data_ptr(), scale, W * H)[0]
            img = fr.download(G.BUF_OUTPUT)[:, :3].astype(np.float64)
            e = np.mean((img - ref) ** 2 / (ref * ref + 1e-2), axis=1)
            assert abs(r - e.mean()) <= 1e-9 * max(r, 1e-30)   # the device reduction agrees with numpy
            rel.append(r)
            med.append(float(np.median(e[fg])))
        fr.close()
        return rel, med

    reuse, reuse_med = run(st, False, 8)
    plain, plain_med = run(G.Settings.make(maxDepth=3, temporalReuse=False, spatialReuse=False), False, 8)
    acc, acc_med = run(st, True, 16)
    print("relMSE reuse", reuse, "median", reuse_med)
    print("relMSE canonical only", plain, "median", plain_med)
    print("relMSE accumulated", acc, "median", acc_med)
    assert np.mean(reuse_med[2:]) < 0.7 * np.mean(plain_med[2:])
    assert acc_med[-1] < 0.5 * acc_med[0]
    scene.close()
    ctx.close()
