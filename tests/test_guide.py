"""The guiding network: its CUDA forward pass, loss gradient and Adam step against the CPU
oracle (oracle/guide_mlp.py, float64 with the same BF16 roundings), and online training that
concentrates the mixture on a target distribution."""
import numpy as np
import pytest

import grisrt as G
from oracle import guide_mlp as M


def _split(p):
    W, b = [], []
    for i, o in M.LAYERS:
        pass
    off = 0
    for i, o in M.LAYERS:
        W.append(p[off:off + i * o].reshape(o, i).astype(np.float64))
        off += i * o
        b.append(p[off:off + o].astype(np.float64))
        off += o
    assert off == len(p)
    return W, b


def _join(W, b):
    return np.concatenate([np.concatenate([w.reshape(-1), bb]) for w, bb in zip(W, b)]).astype(np.float32)


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.exponential(size=n)
    feat = np.concatenate([pos, nrm, wo], axis=1).astype(np.float32)
    return feat, d.astype(np.float32), w.astype(np.float32)


def _params(seed):
    W, b = M.init_params(seed)
    rng = np.random.default_rng(seed + 100)
    b = [rng.normal(0.0, 0.2, bb.shape) for bb in b]
    return W, b


def test_oracle_gradient_matches_finite_differences():
    W, b = _params(3)
    feat, d, w = _inputs(32, 5)
    x = M.encode(feat[:, :3].astype(np.float64), feat[:, 3:6].astype(np.float64), feat[:, 6:9].astype(np.float64))
    loss, dW, db, _ = M.loss_and_grads(W, b, x, d.astype(np.float64), w.astype(np.float64), quantize=False)
    rng = np.random.default_rng(0)
    eps = 1e-6
    for l in range(5):
        for _ in range(4):
            i, j = rng.integers(W[l].shape[0]), rng.integers(W[l].shape[1])
            W[l][i, j] += eps
            lp = M.loss_and_grads(W, b, x, d, w, quantize=False)[0]
            W[l][i, j] -= 2 * eps
            lm = M.loss_and_grads(W, b, x, d, w, quantize=False)[0]
            W[l][i, j] += eps
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - dW[l][i, j]) <= 1e-4 * max(1e-3, abs(fd))


def test_oracle_mixture_sampler_matches_its_density():
    W, b = _params(4)
    feat, _, _ = _inputs(1, 2)
    x = M.encode(feat[:, :3].astype(np.float64), feat[:, 3:6].astype(np.float64), feat[:, 6:9].astype(np.float64))
    out = M.forward(W, b, x, quantize=False)[0]
    rng = np.random.default_rng(1)
    outs = np.repeat(out, 100_000, axis=0)
    dirs = M.sample_mixture(outs, rng.random((100_000, 3)))
    # E[1/p] under the sampler is the sphere's area
    assert abs(np.mean(1.0 / M.mixture_pdf(outs, dirs)) / (4 * np.pi) - 1.0) < 0.02


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1000, 100003])
@pytest.mark.parametrize("tensor_cores", [False, True], ids=["mma_sync", "tcgen05"])
def test_gpu_forward_matches_oracle(tensor_cores, n):
    """Inference by the warp-level mma.sync kernel and by the tcgen05 kernel (128-vertex tiles,
    tensor-memory accumulators): both within the BF16 tolerance of the oracle; n covers partial
    tiles and several tiles per CTA."""
    import torch
    ctx = G.Context(0)
    g = G.Guide(ctx, G.GuideConfig.make(samplesPerFrame=1024, stepsPerFrame=1, tensorCores=tensor_cores))
    W, b = _params(7)
    p = _join(W, b)
    g.set_params(p)
    assert np.array_equal(g.get_params(), p)
    feat, _, _ = _inputs(n, 9)
    tf = torch.from_numpy(feat).cuda()
    to = torch.zeros((n, 40), dtype=torch.float32, device="cuda")
    g.forward(tf.data_ptr(), n, to.data_ptr())
    ctx.sync()
    got = to.cpu().numpy().astype(np.float64)
    x = M.encode(feat[:, :3].astype(np.float64), feat[:, 3:6].astype(np.float64), feat[:, 6:9].astype(np.float64))
    want = M.forward(*_split(p), x, quantize=True)[0][:, :40]
    err = np.abs(got - want)
    scale = np.abs(want).max()
    # the same BF16 roundings on both sides; FP32 against FP64 sums flip a rounding here and there
    assert np.median(err) < 1e-4 * scale
    assert err.max() < 2e-2 * scale
    assert ctx.counters()[3] == 0   # no tensor-core wait gave up
    g.close()
    ctx.close()


TRAIN_KERNELS = [G.GuideConfig.TRAIN_MMA_SYNC, G.GuideConfig.TRAIN_TCGEN05]
TRAIN_IDS = ["mma_sync", "tcgen05"]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3000, 100003, 77])
@pytest.mark.parametrize("kernel", TRAIN_KERNELS, ids=TRAIN_IDS)
def test_gpu_gradient_matches_oracle(kernel, n):
    """The loss gradient by the warp-level mma.sync kernel and by the tcgen05 kernel (128-record
    tiles; dW^T = H^T dZ and dH = dZ W as tensor-core products, the weight gradients accumulated in
    tensor memory across a CTA's tiles, the bias gradients as the ones row of H^T): per layer within
    2e-2 relative L2 of the oracle's float64 gradient with the same BF16 roundings; n covers one
    partial tile, partial tiles at the end and several tiles per CTA."""
    import torch
    ctx = G.Context(0)
    g = G.Guide(ctx, G.GuideConfig.make(samplesPerFrame=1024, stepsPerFrame=1, trainKernel=kernel))
    W, b = _params(11)
    p = _join(W, b)
    g.set_params(p)
    feat, d, w = _inputs(n, 13)
    tf, td, tw = (torch.from_numpy(a).cuda() for a in (feat, d, w))
    grad = torch.zeros(g.n_params, dtype=torch.float32, device="cuda")
    g.gradient(tf.data_ptr(), td.data_ptr(), tw.data_ptr(), n, grad.data_ptr())
    ctx.sync()
    got = grad.cpu().numpy().astype(np.float64)
    x = M.encode(feat[:, :3].astype(np.float64), feat[:, 3:6].astype(np.float64), feat[:, 6:9].astype(np.float64))
    Wq, bq = _split(p)
    _, dW, db, _ = M.loss_and_grads(Wq, bq, x, d.astype(np.float64), w.astype(np.float64), quantize=True)
    want = _join(dW, db).astype(np.float64)
    off = 0
    for l, (i, o) in enumerate(M.LAYERS):
        for part, size in (("W", i * o), ("b", o)):
            a, bb = got[off:off + size], want[off:off + size]
            rel = np.linalg.norm(a - bb) / max(np.linalg.norm(bb), 1e-30)
            assert rel < 2e-2, (l, part, rel)
            off += size
    assert ctx.counters()[3] == 0   # no tensor-core wait gave up
    g.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", TRAIN_KERNELS, ids=TRAIN_IDS)
def test_gpu_adam_step_matches_oracle(kernel):
    import torch
    ctx = G.Context(0)
    lr = 1e-3
    g = G.Guide(ctx, G.GuideConfig.make(samplesPerFrame=1024, stepsPerFrame=1, learningRate=lr, trainKernel=kernel))
    W, b = _params(17)
    p = _join(W, b)
    g.set_params(p)
    n = 2048
    feat, d, w = _inputs(n, 19)
    tf, td, tw = (torch.from_numpy(a).cuda() for a in (feat, d, w))
    grad = torch.zeros(g.n_params, dtype=torch.float32, device="cuda")
    g.gradient(tf.data_ptr(), td.data_ptr(), tw.data_ptr(), n, grad.data_ptr())
    g.train_step(tf.data_ptr(), td.data_ptr(), tw.data_ptr(), n)
    ctx.sync()
    gr = grad.cpu().numpy().astype(np.float64)
    want = [p.astype(np.float64).copy()]
    M.adam(want, [gr], [np.zeros_like(gr)], [np.zeros_like(gr)], 1, lr=lr)
    got = g.get_params().astype(np.float64)
    moved = np.abs(gr) > 1e-6
    assert np.allclose(got[moved], want[0][moved], rtol=0, atol=2e-5)
    assert np.abs(got - p).max() <= 1.001 * lr + 1e-7
    g.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", TRAIN_KERNELS, ids=TRAIN_IDS)
def test_gpu_training_fits_a_target_distribution(kernel):
    """Directions drawn from a position-dependent target (a vMF about a direction that turns with
    x), weight 1: Adam on the loss raises the learned density at the target directions."""
    import torch
    ctx = G.Context(0)
    g = G.Guide(ctx, G.GuideConfig.make(seed=3, samplesPerFrame=1024, stepsPerFrame=1, learningRate=5e-3,
                                        trainKernel=kernel))
    rng = np.random.default_rng(23)
    n = 1 << 14

    def batch():
        pos = rng.random((n, 3))
        ang = pos[:, 0] * np.pi
        mu = np.stack([np.cos(ang), np.sin(ang), np.full(n, 0.3)], axis=1)
        mu /= np.linalg.norm(mu, axis=1, keepdims=True)
        k = 20.0
        u = rng.random((n, 2))
        cz = 1.0 + np.log(u[:, 0] + (1 - u[:, 0]) * np.exp(-2 * k)) / k
        s = np.sqrt(np.maximum(0, 1 - cz * cz))
        t = np.cross(mu, np.array([0.0, 0.0, 1.0]))
        t /= np.linalg.norm(t, axis=1, keepdims=True)
        bb = np.cross(mu, t)
        phi = 2 * np.pi * u[:, 1]
        d = mu * cz[:, None] + t * (s * np.cos(phi))[:, None] + bb * (s * np.sin(phi))[:, None]
        nrm = np.tile([0.0, 0.0, 1.0], (n, 1))
        feat = np.concatenate([pos, nrm, nrm], axis=1).astype(np.float32)
        return feat, d.astype(np.float32), np.ones(n, np.float32), mu

    def mean_logpdf(feat, mu):
        tf = torch.from_numpy(feat).cuda()
        to = torch.zeros((len(feat), 40), dtype=torch.float32, device="cuda")
        g.forward(tf.data_ptr(), len(feat), to.data_ptr())
        ctx.sync()
        return float(np.mean(np.log(M.mixture_pdf(to.cpu().numpy().astype(np.float64), mu))))

    feat0, _, _, mu0 = batch()
    before = mean_logpdf(feat0, mu0)
    for _ in range(300):
        feat, d, w, _ = batch()
        tf, td, tw = (torch.from_numpy(a).cuda() for a in (feat, d, w))
        g.train_step(tf.data_ptr(), td.data_ptr(), tw.data_ptr(), n)
    after = mean_logpdf(feat0, mu0)
    print("mean log pdf at the target's mean direction: before %.3f after %.3f (uniform %.3f, target %.3f)" % (
        before, after, np.log(1 / (4 * np.pi)), np.log(20 / (2 * np.pi))))
    assert after > before + 2.0
    g.close()
    ctx.close()


@pytest.mark.gpu
def test_tcgen05_wait_gives_up_and_reports():
    """The tcgen05 inference with the completion of its matrix products never signalled
    (grisDebugGuideForwardStall): its bounded waits run out, it raises bit 1 of the error word,
    commits once more so that its last bounded wait drains the products in flight (bit 2 stays
    clear: that drain finished), frees its tensor memory and returns; the context then runs an
    ordinary forward correctly."""
    import time
    import torch
    ctx = G.Context(0)
    g = G.Guide(ctx, G.GuideConfig.make(samplesPerFrame=1024, stepsPerFrame=1, tensorCores=True))
    p = _join(*_params(3))
    g.set_params(p)
    n = 300
    feat, _, _ = _inputs(n, 4)
    tf = torch.from_numpy(feat).cuda()
    to = torch.zeros((n, 40), dtype=torch.float32, device="cuda")
    lib = G.load()
    t0 = time.time()
    ctx.check(lib.grisDebugGuideForwardStall(ctx.h, g.h, tf.data_ptr(), n, to.data_ptr()), "stall")
    rc = lib.grisSync(ctx.h)
    assert rc == -5, rc                              # GRIS_ERR_DEVICE_FAULT
    assert time.time() - t0 < 10.0
    c = ctx.counters(reset=True)
    assert c[3] & 2
    assert not (c[3] & 4)                            # the drain after the timeout completed
    g.forward(tf.data_ptr(), n, to.data_ptr())       # the context is still usable
    ctx.sync()
    x = M.encode(feat[:, :3].astype(np.float64), feat[:, 3:6].astype(np.float64), feat[:, 6:9].astype(np.float64))
    want = M.forward(*_split(p), x, quantize=True)[0][:, :40]
    got = to.cpu().numpy().astype(np.float64)
    assert np.median(np.abs(got - want)) < 1e-4 * np.abs(want).max()
    assert ctx.counters()[3] == 0
    g.close()
    ctx.close()
