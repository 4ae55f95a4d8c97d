"""grisPassRenderNoAlloc: the GRIS pass for callers that cannot allocate device memory while
they render (a host callback or plugin that must not call cudaMalloc, a process whose device
allocator belongs to another framework). Its scratch lives in a static device array of the
library, so its results must equal those of grisPassRender with a zero-filled temporary
reservoir buffer, bit for bit, call after call.

Collected last on purpose (file name), so that a run stopping at the first failure has run
every other test first."""
import ctypes

import numpy as np
import pytest

import grisrt as G

pytestmark = pytest.mark.gpu

GRIS_ERR_TOO_LARGE = -6


def test_no_alloc_pass_matches_allocating_pass_on_consecutive_calls():
    import torch
    lib = G.load()
    ctx = G.Context(0)
    hs = G.HostScene(0, seed=4)
    W, H = 64, 48
    assert W * H <= G.NOALLOC_MAX_PIXELS
    cams, prevs = G.sequence_cameras(hs, 2, W, H, seed=9)
    st = G.Settings.make(maxDepth=4, spatialRadius=30.0)
    scene = G.Scene(ctx, hs)
    n = W * H
    z = lambda *shape, dt=torch.int32: torch.zeros(shape, dtype=dt, device="cuda")
    dn = [z(n, 4, dt=torch.float32) for _ in range(2)]
    am = [z(n, 2) for _ in range(2)]
    mv = z(n, 2, dt=torch.int16)
    a_resv, b_resv = [z(n, 24) for _ in range(2)], [z(n, 24) for _ in range(2)]
    a_out, b_out = z(n, 4, dt=torch.float32), z(n, 4, dt=torch.float32)
    a_temp = z(n, 24)
    torch.cuda.synchronize()
    for f in range(2):
        j = f & 1
        gb = G.GBufferBindings(W, H, dn[j].data_ptr(), am[j].data_ptr(), mv.data_ptr())
        ctx.check(lib.grisPassGBuffer(ctx.h, scene.h, ctypes.byref(gb), ctypes.byref(cams[f])), "grisPassGBuffer")
        ctx.sync()
        # the allocating pass, with a zero-filled temporary reservoir buffer
        a_temp.zero_()
        torch.cuda.synchronize()
        ba = G.PassBindings(W, H, dn[j].data_ptr(), dn[j ^ 1].data_ptr(), am[j].data_ptr(), am[j ^ 1].data_ptr(),
                            mv.data_ptr(), a_resv[j].data_ptr(), a_resv[j ^ 1].data_ptr(), a_temp.data_ptr(),
                            a_out.data_ptr())
        ctx.check(lib.grisPassRender(ctx.h, scene.h, ctypes.byref(ba), ctypes.byref(cams[f]), ctypes.byref(prevs[f]),
                                     ctypes.byref(st), 7), "grisPassRender")
        ctx.sync()
        # the allocation-free pass on the same inputs, same stream
        bb = G.PassBindings(W, H, dn[j].data_ptr(), dn[j ^ 1].data_ptr(), am[j].data_ptr(), am[j ^ 1].data_ptr(),
                            mv.data_ptr(), b_resv[j].data_ptr(), b_resv[j ^ 1].data_ptr(), None, b_out.data_ptr())
        dev_before = torch.cuda.current_device()
        rc = lib.grisPassRenderNoAlloc(scene.h, ctypes.byref(bb), ctypes.byref(cams[f]), ctypes.byref(prevs[f]),
                                       ctypes.byref(st), ctx.stream())
        assert rc == 0, rc
        assert torch.cuda.current_device() == dev_before   # the caller's current device is given back
        ctx.sync()
        # no device-side error (traversal stack limit) was raised; reading clears the word
        word = ctypes.c_uint64(123)
        assert lib.grisNoAllocReadError(0, ctx.stream(), ctypes.byref(word)) == 0
        assert word.value == 0
        ra, rb = a_resv[j].cpu().numpy(), b_resv[j].cpu().numpy()
        assert ra.tobytes() == rb.tobytes(), "call %d: reservoirs differ" % f
        assert a_out.cpu().numpy().tobytes() == b_out.cpu().numpy().tobytes(), "call %d: radiance differs" % f
        valid = ra.view(G.RESERVOIR)["instanceIdx"] != G.INVALID_HIT
        assert valid.mean() > 0.5   # the comparison is not between two empty frames
    assert b_out.cpu().numpy()[:, :3].max() > 0.0
    scene.close()
    ctx.close()


def test_no_alloc_pass_rejects_frames_beyond_its_limit():
    import torch
    lib = G.load()
    ctx = G.Context(0)
    hs = G.HostScene(0, seed=4)
    scene = G.Scene(ctx, hs)
    W, H = 512, 256   # 131072 pixels > 65536
    cam = hs.camera(0, 1, W, H)
    st = G.Settings.make()
    t = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = t.data_ptr()
    b = G.PassBindings(W, H, p, p, p, p, p, p, p, None, p)
    rc = lib.grisPassRenderNoAlloc(scene.h, ctypes.byref(b), ctypes.byref(cam), ctypes.byref(cam), ctypes.byref(st), None)
    assert rc == GRIS_ERR_TOO_LARGE
    assert not t.any()   # nothing was launched
    scene.close()
    ctx.close()
