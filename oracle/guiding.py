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
  network    256 -> 64 -> 64 -> 64 -> 64 -> 64, ReLU after the first four
             layers; BF16 weights and activations, FP32 accumulation
  output     8 anisotropic lobes, 8 numbers each (a, mx, my, mz, b, ux, uy,
             uz): weight softmax(a), mean direction mu = normalize(m),
             isotropic precision s = exp(clip(b, -3, 8)), and the tangent
             projection pu = u - (u . mu) mu of an anisotropy vector
  lobe       a 2D Gaussian in the plane tangent to the sphere at mu, mapped to
             the sphere by gnomonic projection (w = normalize(mu + x)): with
             c = mu . w > 0, v = w / c - mu, the precision s I + pu pu^T
             (eigenvalues s and s + |pu|^2) and Q = s |v|^2 + (pu . v)^2,
             p(w) = sqrt(s (s + |pu|^2)) / (2 pi) exp(-Q / 2) / c^3
             (the 1 / c^3 is the projection's area change); 0 where c <= 0
  density    q(w) = (1 - eps) sum_i pi_i p_i(w) + eps / (4 pi), eps = 0.02: a
             uniform component keeps q > 0 everywhere
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
LOBE_OUT = 8  # raw outputs per lobe: a, m (3), b, u (3)
N_OUT = LOBE_OUT * LOBES
LAYERS = [(N_IN, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, N_OUT)]
B_MIN, B_MAX = -3.0, 8.0
EPS_UNIFORM = 0.02   # probability of the uniform component
C_MIN = 1e-4         # lobes are zero where mu . w <= C_MIN


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


def mixture(raw: np.ndarray) -> dict:
    """raw (N, 64) -> lobe weights pi (N,8), unit means mu (N,8,3), isotropic
    precisions s (N,8), tangent anisotropy pu (N,8,3), and what the gradient
    needs: the raw u, |m| and the mask of b inside its clip range."""
    r = raw.reshape(-1, LOBES, LOBE_OUT)
    a = r[:, :, 0]
    a = a - a.max(axis=1, keepdims=True)
    e = np.exp(a)
    pi = e / e.sum(axis=1, keepdims=True)
    m = r[:, :, 1:4]
    norm = np.linalg.norm(m, axis=2, keepdims=True)
    mu = np.where(norm > 1e-12, m / np.maximum(norm, 1e-30), np.array([0.0, 0.0, 1.0]))
    b = r[:, :, 4]
    inside = (b > B_MIN) & (b < B_MAX)
    s = np.exp(np.clip(b, B_MIN, B_MAX))
    u = r[:, :, 5:8]
    pu = u - np.einsum("nlk,nlk->nl", u, mu)[:, :, None] * mu
    return {"pi": pi, "mu": mu, "s": s, "pu": pu, "u": u, "norm": norm[:, :, 0], "inside": inside}


def lobe_terms(mx: dict, w: np.ndarray) -> dict:
    """Per lobe at unit directions w (N, 3): c, v, |v|^2, pu . v, and log p
    (-inf where c <= C_MIN)."""
    mu, s, pu = mx["mu"], mx["s"], mx["pu"]
    c = np.einsum("nlk,nk->nl", mu, w)
    valid = c > C_MIN
    cs = np.where(valid, c, 1.0)
    v = w[:, None, :] / cs[:, :, None] - mu
    v2 = np.einsum("nlk,nlk->nl", v, v)
    d = np.einsum("nlk,nlk->nl", pu, v)
    p2 = np.einsum("nlk,nlk->nl", pu, pu)
    q = s * v2 + d * d
    logp = 0.5 * np.log(s) + 0.5 * np.log(s + p2) - np.log(2.0 * np.pi) - 0.5 * q - 3.0 * np.log(cs)
    logp = np.where(valid, logp, -np.inf)
    return {"c": cs, "valid": valid, "v": v, "v2": v2, "d": d, "p2": p2, "logp": logp}


def mixture_pdf(raw: np.ndarray, w: np.ndarray) -> np.ndarray:
    mx = mixture(raw)
    t = lobe_terms(mx, w)
    return (1.0 - EPS_UNIFORM) * (mx["pi"] * np.exp(t["logp"])).sum(axis=1) + EPS_UNIFORM / (4.0 * np.pi)


def sample_mixture(raw: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Directions drawn from the mixture of each row of raw, u (N, 4) uniform
    in [0, 1): the uniform component with probability eps, else a lobe by
    weight, then the tangent-plane Gaussian (Box-Muller) projected."""
    mx = mixture(raw)
    n = len(raw)
    out = np.zeros((n, 3))
    for i in range(n):
        if u[i, 0] < EPS_UNIFORM:
            z = 1.0 - 2.0 * u[i, 1]
            ph = 2.0 * np.pi * u[i, 2]
            rr = np.sqrt(max(0.0, 1.0 - z * z))
            out[i] = (rr * np.cos(ph), rr * np.sin(ph), z)
            continue
        x = (u[i, 0] - EPS_UNIFORM) / (1.0 - EPS_UNIFORM)
        lobe = min(int(np.searchsorted(np.cumsum(mx["pi"][i]), x, side="right")), LOBES - 1)
        mu, s, pu = mx["mu"][i, lobe], mx["s"][i, lobe], mx["pu"][i, lobe]
        p2 = pu @ pu
        if p2 > 1e-20:
            e2 = pu / np.sqrt(p2)
        else:
            e2 = np.cross(mu, [1.0, 0.0, 0.0] if abs(mu[0]) < 0.9 else [0.0, 1.0, 0.0])
            e2 /= np.linalg.norm(e2)
        e1 = np.cross(mu, e2)
        r = np.sqrt(-2.0 * np.log(max(u[i, 1], 1e-300)))
        g1, g2 = r * np.cos(2.0 * np.pi * u[i, 2]), r * np.sin(2.0 * np.pi * u[i, 2])
        x = g1 / np.sqrt(s) * e1 + g2 / np.sqrt(s + p2) * e2
        d = mu + x
        out[i] = d / np.linalg.norm(d)
    return out


def loss_grad(raw: np.ndarray, w: np.ndarray, weight: np.ndarray):
    """Loss = mean(-weight * log q(w)); returns (loss, dLoss/draw (N, 64))."""
    n = len(raw)
    mx = mixture(raw)
    t = lobe_terms(mx, w)
    p = np.exp(t["logp"])
    q = (1.0 - EPS_UNIFORM) * (mx["pi"] * p).sum(axis=1) + EPS_UNIFORM / (4.0 * np.pi)
    loss = float(np.mean(-weight * np.log(q)))
    resp = (1.0 - EPS_UNIFORM) * mx["pi"] * p / q[:, None]       # responsibilities of the lobes
    coef = (-weight / n)[:, None]                                  # d loss / d log q
    g = np.zeros((n, LOBES, LOBE_OUT))
    g[:, :, 0] = coef * (resp - mx["pi"] * resp.sum(axis=1, keepdims=True))
    mu, s, pu, u = mx["mu"], mx["s"], mx["pu"], mx["u"]
    c, v, v2, d, p2 = t["c"], t["v"], t["v2"], t["d"], t["p2"]
    cr = (coef * resp)[:, :, None]
    sp2 = s + p2
    # b (through s = exp(b) inside the clip range)
    g[:, :, 4] = coef * resp * (0.5 + 0.5 * s / sp2 - 0.5 * s * v2) * mx["inside"]
    # u: d|pu|^2/du = 2 pu, d(pu . v)/du = v (v is tangent)
    g[:, :, 5:8] = cr * (pu / sp2[:, :, None] - d[:, :, None] * v)
    # mu: through c = mu . w, v = w / c - mu and pu = u - (u . mu) mu
    um = np.einsum("nlk,nlk->nl", u, mu)[:, :, None]
    vw = np.einsum("nlk,nk->nl", v, w)[:, :, None]
    pw = np.einsum("nlk,nk->nl", pu, w)[:, :, None]
    wc2 = w[:, None, :] / (c * c)[:, :, None]
    gmu = (-um * pu / sp2[:, :, None]
           + s[:, :, None] * (vw * wc2 + v)
           + d[:, :, None] * (um * v + pw * wc2 + pu)
           - 3.0 * w[:, None, :] / c[:, :, None])
    gmu = gmu - np.einsum("nlk,nlk->nl", gmu, mu)[:, :, None] * mu
    norm = np.maximum(mx["norm"], 1e-30)[:, :, None]
    g[:, :, 1:4] = cr * gmu / norm * (mx["norm"] > 1e-12)[:, :, None]
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
