"""CPU restatement (FP64, numpy) of the learned path-guiding model.

Test infrastructure: imported only by tests/ as the checker of the GPU
guiding kernels (muon_gb300/csrc/guide.cu). The reference renderer has no
learned component, so this file restates the model the GPU implements, not
reference code:

  features   8 numbers in [0, 1]: position in the scene box (3), shading
             normal as (theta / pi, phi / 2pi + 1/2) (2), outgoing direction
             in the same form (2), roughness (1)
  encoding   one-blob (Mueller et al., "Neural Importance Sampling", 2019):
             each feature s -> 32 bins, bin k = exp(-(s - (k + 1/2) / 32)^2 /
             (2 sigma^2)), sigma = 1/32; 256 inputs
  network    256 -> 64 -> 64 -> 64 -> 64 -> 40, ReLU after the first four
             layers; BF16 weights and activations, FP32 accumulation
  output     8 von Mises-Fisher lobes, 5 numbers each (a, mx, my, mz, b):
             weight softmax(a), mean direction normalize(m), concentration
             kappa = exp(clip(b, -3, 8))
  density    q(w) = sum_i pi_i kappa_i / (2 pi (1 - exp(-2 kappa_i)))
                    * exp(kappa_i (mu_i . w - 1))
  loss       -weight * log q(w) per sample (the KL-divergence estimator of
             Mueller et al. 2019, weight = target / sampling density), mean
             over the batch; Adam (Kingma and Ba, 2015).
"""
from __future__ import annotations

import numpy as np

BINS = 32
SIGMA = 1.0 / BINS
N_FEATURES = 8
N_IN = N_FEATURES * BINS
WIDTH = 64
LOBES = 8
N_OUT = 5 * LOBES
LAYERS = [(N_IN, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, N_OUT)]
B_MIN, B_MAX = -3.0, 8.0


def bf16(x: np.ndarray) -> np.ndarray:
    """Rounds float values to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(x, dtype=np.float32).copy()
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    out = (u & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    nan = np.isnan(f)
    out[nan] = np.nan
    return out.astype(np.float64)


def one_blob(features: np.ndarray) -> np.ndarray:
    """(N, 8) features in [0, 1] -> (N, 256) one-blob encoding."""
    f = np.clip(np.asarray(features, dtype=np.float64), 0.0, 1.0)
    centres = (np.arange(BINS) + 0.5) / BINS
    d = f[:, :, None] - centres[None, None, :]
    return np.exp(-d * d / (2.0 * SIGMA * SIGMA)).reshape(len(f), N_IN)


def init_params(seed: int) -> list[tuple[np.ndarray, np.ndarray]]:
    """He-uniform weights (in, out) and zero biases; the GPU initialises with
    the same recipe from its own generator, so tests pass weights across."""
    rng = np.random.default_rng(seed)
    params = []
    for fan_in, fan_out in LAYERS:
        lim = np.sqrt(6.0 / fan_in)
        params.append((rng.uniform(-lim, lim, size=(fan_in, fan_out)), np.zeros(fan_out)))
    return params


def forward(params, features: np.ndarray, bf16_round: bool = True):
    """Returns (outputs (N, 40), activations list) with BF16 rounding of the
    GEMM operands when bf16_round (the GPU's arithmetic up to accumulation
    order)."""
    r = bf16 if bf16_round else (lambda x: np.asarray(x, dtype=np.float64))
    h = r(one_blob(features))
    acts = [h]
    zs = []
    for li, (w, b) in enumerate(params):
        z = h @ r(w) + b
        zs.append(z)
        if li < len(params) - 1:
            h = r(np.maximum(z, 0.0))
            acts.append(h)
        else:
            h = z
    return h, acts, zs


def mixture(raw: np.ndarray):
    """raw (N, 40) -> (pi (N,8), mu (N,8,3), kappa (N,8), b_clipped_mask)."""
    r = raw.reshape(-1, LOBES, 5)
    a = r[:, :, 0]
    a = a - a.max(axis=1, keepdims=True)
    e = np.exp(a)
    pi = e / e.sum(axis=1, keepdims=True)
    m = r[:, :, 1:4]
    norm = np.linalg.norm(m, axis=2, keepdims=True)
    mu = np.where(norm > 1e-12, m / np.maximum(norm, 1e-30), np.array([0.0, 0.0, 1.0]))
    b = r[:, :, 4]
    inside = (b > B_MIN) & (b < B_MAX)
    kappa = np.exp(np.clip(b, B_MIN, B_MAX))
    return pi, mu, kappa, inside


def vmf_log_pdf(mu: np.ndarray, kappa: np.ndarray, w: np.ndarray) -> np.ndarray:
    """log vMF density for lobes (N, L) at unit directions w (N, 3)."""
    cos = np.einsum("nlk,nk->nl", mu, w)
    return (np.log(kappa) - np.log(2.0 * np.pi) - np.log1p(-np.exp(-2.0 * kappa)) + kappa * (cos - 1.0))


def mixture_pdf(raw: np.ndarray, w: np.ndarray) -> np.ndarray:
    pi, mu, kappa, _ = mixture(raw)
    return (pi * np.exp(vmf_log_pdf(mu, kappa, w))).sum(axis=1)


def loss_grad(raw: np.ndarray, w: np.ndarray, weight: np.ndarray):
    """Loss = mean(-weight * log q(w)); returns (loss, dLoss/draw (N, 40))."""
    n = len(raw)
    r = raw.reshape(n, LOBES, 5)
    pi, mu, kappa, inside = mixture(raw)
    logf = vmf_log_pdf(mu, kappa, w)
    f = np.exp(logf)
    q = (pi * f).sum(axis=1)
    loss = float(np.mean(-weight * np.log(q)))
    resp = pi * f / q[:, None]                         # responsibilities
    coef = (-weight / n)[:, None]                      # d loss / d log q
    g = np.zeros_like(r)
    g[:, :, 0] = coef * (resp - pi)                    # softmax
    m = r[:, :, 1:4]
    norm = np.maximum(np.linalg.norm(m, axis=2, keepdims=True), 1e-30)
    cos = np.einsum("nlk,nk->nl", mu, w)
    dlog_dmu = kappa[:, :, None] * w[:, None, :]       # d(kappa mu.w)/dmu
    # through mu = m / |m|: (I - mu mu^T) / |m|
    proj = dlog_dmu - (np.einsum("nlk,nlk->nl", dlog_dmu, mu))[:, :, None] * mu
    g[:, :, 1:4] = (coef * resp)[:, :, None] * proj / norm
    e2 = np.exp(-2.0 * kappa)
    dlog_dkappa = 1.0 / kappa - 2.0 * e2 / (1.0 - e2) + (cos - 1.0)
    g[:, :, 4] = coef * resp * dlog_dkappa * kappa * inside
    return loss, g.reshape(n, N_OUT)


def backward(params, acts, zs, dout):
    """Gradients of the loss for every (W, b) given dLoss/doutput."""
    grads = [None] * len(params)
    d = dout
    for li in range(len(params) - 1, -1, -1):
        w, _ = params[li]
        grads[li] = (acts[li].T @ d, d.sum(axis=0))
        if li > 0:
            d = (d @ w.T) * (zs[li - 1] > 0)
    return grads


def adam_step(params, grads, state, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update in place; state = {'t': int, 'm': [...], 'v': [...]}."""
    if not state:
        state["t"] = 0
        state["m"] = [(np.zeros_like(w), np.zeros_like(b)) for w, b in params]
        state["v"] = [(np.zeros_like(w), np.zeros_like(b)) for w, b in params]
    state["t"] += 1
    t = state["t"]
    out = []
    for i, ((w, b), (gw, gb)) in enumerate(zip(params, grads)):
        (mw, mb), (vw, vb) = state["m"][i], state["v"][i]
        mw = beta1 * mw + (1 - beta1) * gw
        mb = beta1 * mb + (1 - beta1) * gb
        vw = beta2 * vw + (1 - beta2) * gw * gw
        vb = beta2 * vb + (1 - beta2) * gb * gb
        state["m"][i], state["v"][i] = (mw, mb), (vw, vb)
        c1, c2 = 1 - beta1 ** t, 1 - beta2 ** t
        w = w - lr * (mw / c1) / (np.sqrt(vw / c2) + eps)
        b = b - lr * (mb / c1) / (np.sqrt(vb / c2) + eps)
        out.append((w, b))
    return out


def features_of(pos, normal, wo, roughness, lo, hi):
    """The feature vector of a shading point (see the module docstring)."""
    def sph(v):
        v = np.asarray(v, dtype=np.float64)
        theta = np.arccos(np.clip(v[..., 2], -1.0, 1.0)) / np.pi
        phi = np.arctan2(v[..., 1], v[..., 0]) / (2.0 * np.pi) + 0.5
        return np.stack([theta, phi], axis=-1)

    p = (np.asarray(pos, dtype=np.float64) - lo) / np.maximum(np.asarray(hi) - lo, 1e-30)
    return np.concatenate([np.clip(p, 0, 1), sph(normal), sph(wo), np.asarray(roughness)[..., None]], axis=-1)


def flatten(params) -> np.ndarray:
    """(W, b) per layer -> the library's flat FP32 layout (W [in][out], then b)."""
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in params]).astype(np.float32)


def unflatten(flat: np.ndarray):
    out, off = [], 0
    for fan_in, fan_out in LAYERS:
        w = np.asarray(flat[off:off + fan_in * fan_out], dtype=np.float64).reshape(fan_in, fan_out)
        off += fan_in * fan_out
        b = np.asarray(flat[off:off + fan_out], dtype=np.float64)
        off += fan_out
        out.append((w, b))
    return out


N_PARAMS = sum(a * b + b for a, b in LAYERS)
