"""CPU oracle of the guiding network (float64 numpy).

TEST INFRASTRUCTURE: only tests/ import it, as the checker of the CUDA guide kernels.

The proposal is a mixture of 8 von Mises-Fisher lobes over world-space directions, predicted
per path vertex by an MLP:
  input   the vertex position normalised to the scene box (each coordinate p in [0,1]) encoded
          as sin(2^k pi p), cos(2^k pi p) for k = 0..11 (72 values, ordered per coordinate: the
          12 sines then the 12 cosines of x, then of y, then of z), the shading normal (3) and
          the direction towards the previous vertex wo (3): 78 values, zero-padded to 80;
  layers  80 -> 64 -> 64 -> 64 -> 64 (ReLU) -> 48 (linear; the first 40 used), weights W[out][in]
          and biases, BF16 weights and activations with FP32 accumulation on the device;
  output  per lobe j (values 5j..5j+4): a direction m (3) -> mu = m / |m|, kappa = exp(clamp(k,
          -4, 7)), a logit -> pi = softmax(logits).
vMF density: kappa / (2 pi (1 - exp(-2 kappa))) * exp(kappa (mu . w - 1)).
Training loss over a batch (Mueller et al. 2019, KL divergence by Monte Carlo): with weights
w_i = target_i / q_i (target = the luminance of the sampled direction's contribution f cos L_in,
q = the pdf it was sampled with), loss = -sum_i w_i log p(w_i | x_i) / sum_i w_i.
"""
import numpy as np

IN, HID, OUT, LOBES = 80, 64, 48, 8
LAYERS = [(IN, HID), (HID, HID), (HID, HID), (HID, HID), (HID, OUT)]
FREQS = 12
KMIN, KMAX = -4.0, 7.0


def encode(pos01, normal, wo):
    """pos01: [n,3] in [0,1]; returns [n,80] float64."""
    n = len(pos01)
    x = np.zeros((n, IN))
    k = 2.0 ** np.arange(FREQS)
    for c in range(3):
        a = np.pi * pos01[:, c:c + 1] * k[None, :]
        x[:, c * 24:c * 24 + 12] = np.sin(a)
        x[:, c * 24 + 12:c * 24 + 24] = np.cos(a)
    x[:, 72:75] = normal
    x[:, 75:78] = wo
    return x


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def init_params(seed=0):
    """Uniform(-sqrt(6/(in+out)), +) weights (Glorot), zero biases; kappa biases start at 1."""
    rng = np.random.default_rng(seed)
    W, b = [], []
    for i, o in LAYERS:
        lim = np.sqrt(6.0 / (i + o))
        W.append(rng.uniform(-lim, lim, (o, i)))
        b.append(np.zeros(o))
    return W, b


def forward(W, b, x, quantize=True):
    """Returns (output [n,48], activations list: inputs of each layer, pre-activations)."""
    q = bf16 if quantize else (lambda a: a)
    acts, pres = [], []
    h = q(x)
    for l in range(5):
        acts.append(h)
        z = h @ q(W[l]).T + b[l]
        pres.append(z)
        if l < 4:
            h = q(np.maximum(z, 0.0))
        else:
            h = z
    return h, acts, pres


def lobes(out):
    """(mu [n,8,3], kappa [n,8], pi [n,8], aux) from the raw output [n,48]."""
    o = out[:, :40].reshape(-1, LOBES, 5)
    m = o[:, :, 0:3]
    norm = np.linalg.norm(m, axis=2)
    mu = m / np.maximum(norm, 1e-12)[:, :, None]
    kr = np.clip(o[:, :, 3], KMIN, KMAX)
    kappa = np.exp(kr)
    lg = o[:, :, 4]
    lg = lg - lg.max(axis=1, keepdims=True)
    e = np.exp(lg)
    pi = e / e.sum(axis=1, keepdims=True)
    return mu, kappa, pi, (m, norm, o[:, :, 3])


def vmf_log(mu, kappa, w):
    """log vMF(w) per lobe; w [n,3]."""
    c = np.einsum("njk,nk->nj", mu, w)
    return np.log(kappa) - np.log(2.0 * np.pi) - np.log1p(-np.exp(-2.0 * kappa)) + kappa * (c - 1.0)


def mixture_pdf(out, w):
    mu, kappa, pi, _ = lobes(out)
    return np.sum(pi * np.exp(vmf_log(mu, kappa, w)), axis=1)


def loss_and_grad_out(out, w_dir, weight):
    """loss = -sum weight log p / sum weight; returns (loss, dloss/dout [n,48])."""
    n = len(out)
    mu, kappa, pi, (m, norm, kraw) = lobes(out)
    lv = vmf_log(mu, kappa, w_dir)
    lp = np.log(pi) + lv
    mx = lp.max(axis=1, keepdims=True)
    logp = (mx[:, 0] + np.log(np.exp(lp - mx).sum(axis=1)))
    r = np.exp(lp - logp[:, None])                     # responsibilities
    sw = weight.sum()
    loss = -np.sum(weight * logp) / sw
    g = -(weight / sw)[:, None]                        # dloss/dlogp
    d = np.zeros((n, LOBES, 5))
    # logits
    d[:, :, 4] = g * (r - pi)
    # log vMF_j = log k - log 2pi - log(1 - e^{-2k}) + k (mu.w - 1)
    c = np.einsum("njk,nk->nj", mu, w_dir)
    e2 = np.exp(-2.0 * kappa)
    dlv_dk = 1.0 / kappa - 2.0 * e2 / (1.0 - e2) + (c - 1.0)
    inside = (kraw > KMIN) & (kraw < KMAX)
    d[:, :, 3] = g * r * dlv_dk * kappa * inside
    # mu = m/|m|: dlv/dm = kappa (w - (mu.w) mu) / |m|
    dmu = kappa[:, :, None] * w_dir[:, None, :]
    dm = (dmu - np.sum(dmu * mu, axis=2, keepdims=True) * mu) / np.maximum(norm, 1e-12)[:, :, None]
    d[:, :, 0:3] = (g * r)[:, :, None] * dm
    dout = np.zeros((n, OUT))
    dout[:, :40] = d.reshape(n, 40)
    return loss, dout


def backward(W, acts, pres, dout, quantize=True):
    """Gradients of the weights and biases given dloss/dout (activations as in forward)."""
    q = bf16 if quantize else (lambda a: a)
    dW, db = [None] * 5, [None] * 5
    dz = dout
    for l in range(4, -1, -1):
        dW[l] = dz.T @ acts[l]
        db[l] = dz.sum(axis=0)
        if l > 0:
            dh = dz @ q(W[l])
            dz = dh * (pres[l - 1] > 0.0)
    return dW, db


def loss_and_grads(W, b, x, w_dir, weight, quantize=True):
    out, acts, pres = forward(W, b, x, quantize)
    loss, dout = loss_and_grad_out(out, w_dir, weight)
    dW, db = backward(W, acts, pres, dout, quantize)
    return loss, dW, db, out


def adam(params, grads, m, v, t, lr=1e-3, b1=0.9, b2=0.99, eps=1e-8):
    """One Adam step (bias-corrected), in place; t is the 1-based step count."""
    for p, g, mm, vv in zip(params, grads, m, v):
        mm *= b1
        mm += (1.0 - b1) * g
        vv *= b2
        vv += (1.0 - b2) * g * g
        mh = mm / (1.0 - b1 ** t)
        vh = vv / (1.0 - b2 ** t)
        p -= lr * mh / (np.sqrt(vh) + eps)


def sample_mixture(out, u):
    """Directions from the mixture, u [n,3] uniforms: lobe by u0 over pi, then the vMF by (u1, u2)
    (w = 1 + log(u1 + (1 - u1) e^{-2k}) / k, phi = 2 pi u2, around mu)."""
    mu, kappa, pi, _ = lobes(out)
    n = len(out)
    cdf = np.cumsum(pi, axis=1)
    j = np.minimum((u[:, 0:1] > cdf).sum(axis=1), LOBES - 1)
    m = mu[np.arange(n), j]
    k = kappa[np.arange(n), j]
    wz = 1.0 + np.log(u[:, 1] + (1.0 - u[:, 1]) * np.exp(-2.0 * k)) / k
    wz = np.clip(wz, -1.0, 1.0)
    s = np.sqrt(np.maximum(0.0, 1.0 - wz * wz))
    phi = 2.0 * np.pi * u[:, 2]
    t = np.where(np.abs(m[:, 2:3]) > 0.999, np.array([[0.0, 1.0, 0.0]]), np.array([[0.0, 0.0, 1.0]]))
    bb = np.cross(m, t)
    bb /= np.linalg.norm(bb, axis=1, keepdims=True)
    tt = np.cross(bb, m)
    return tt * (s * np.cos(phi))[:, None] + bb * (s * np.sin(phi))[:, None] + m * wz[:, None]
