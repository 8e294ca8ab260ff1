"""Learned path guiding: the network, its training and the guided estimator.

The oracle (oracle/guiding.py, FP64 numpy) is pinned first by finite
differences. The GPU's tensor-core forward pass must match the oracle's
forward pass with the same BF16 rounding of weights and activations to the
accuracy BF16 allows; its FP32 training gradients must match the oracle's
FP64 gradients for the same parameters; training must lower the loss on a
known target; guided renders must converge to the same image as plain ones
(the estimator is unbiased whatever the network predicts).
"""
import numpy as np
import pytest

import muon_gb300 as m
from muon_gb300 import native, scenes
from oracle import guiding as G


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n = 12
    feat = rng.uniform(0, 1, (n, 8))
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    wt = rng.uniform(0.1, 2.0, n)
    params = G.init_params(3)
    out, acts, zs = G.forward(params, feat, bf16_round=False)
    loss, dout = G.loss_grad(out, w, wt)
    grads = G.backward(params, acts, zs, dout)
    eps = 1e-6
    for j in range(G.N_OUT):
        o2 = out.copy()
        o2[5, j] += eps
        fd = (G.loss_grad(o2, w, wt)[0] - loss) / eps
        assert abs(fd - dout[5, j]) <= 1e-5 * max(1.0, abs(fd))
    for li, (a, b) in [(0, (17, 3)), (1, (5, 60)), (3, (40, 2)), (4, (63, 39))]:
        p2 = [(x.copy(), y.copy()) for x, y in params]
        p2[li][0][a, b] += eps
        o3, _, _ = G.forward(p2, feat, bf16_round=False)
        fd = (G.loss_grad(o3, w, wt)[0] - loss) / eps
        assert abs(fd - grads[li][0][a, b]) <= 1e-5 * max(1.0, abs(fd))


def test_oracle_lobe_gradients_match_finite_differences():
    """The mixture loss gradient of every raw output, with lobes aimed near
    the sample directions so that every term is exercised."""
    rng = np.random.default_rng(0)
    n = 12
    raw = rng.normal(0, 1, (n, G.N_OUT))
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    raw.reshape(n, G.LOBES, G.LOBE_OUT)[:, :, 1:4] += 2.0 * w[:, None, :]
    wt = rng.uniform(0.1, 2.0, n)
    _, g = G.loss_grad(raw, w, wt)
    eps = 1e-6
    for i in range(n):
        for j in range(G.N_OUT):
            r2, r3 = raw.copy(), raw.copy()
            r2[i, j] += eps
            r3[i, j] -= eps
            fd = (G.loss_grad(r2, w, wt)[0] - G.loss_grad(r3, w, wt)[0]) / (2 * eps)
            assert abs(fd - g[i, j]) <= 1e-5 * max(1e-2, abs(fd)), (i, j, fd, g[i, j])


def _sphere_points(rng, n):
    z = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(ph), r * np.sin(ph), z], 1)


def _strong_mixture(rng):
    raw = rng.normal(0, 1.5, G.N_OUT)
    raw.reshape(G.LOBES, G.LOBE_OUT)[:, 4] += 2.0      # concentrated
    raw.reshape(G.LOBES, G.LOBE_OUT)[:, 5:8] *= 8.0    # strongly anisotropic
    return raw


def test_oracle_mixture_density_integrates_to_one():
    rng = np.random.default_rng(1)
    for _ in range(3):
        raw = _strong_mixture(rng)
        wu = _sphere_points(rng, 1_000_000)
        q = G.mixture_pdf(np.broadcast_to(raw, (len(wu), G.N_OUT)), wu)
        total = 4 * np.pi * q.mean()
        se = 4 * np.pi * q.std() / np.sqrt(len(wu))
        assert abs(total - 1.0) <= 4 * se + 1e-3, (total, se)


def test_oracle_sampler_draws_from_the_density():
    """Moments of sampled directions against the same moments of the density
    (uniform sphere points weighted by q): z-scores within 4."""
    rng = np.random.default_rng(2)
    for _ in range(2):
        raw = _strong_mixture(rng)
        ws = G.sample_mixture(np.broadcast_to(raw, (40000, G.N_OUT)), rng.random((40000, 4)))
        wu = _sphere_points(rng, 1_000_000)
        qu = G.mixture_pdf(np.broadcast_to(raw, (len(wu), G.N_OUT)), wu)
        for f in (lambda v: v[:, 0], lambda v: v[:, 1], lambda v: v[:, 2], lambda v: v[:, 0] * v[:, 1],
                  lambda v: v[:, 2] ** 2, lambda v: v[:, 0] * v[:, 2]):
            a, sa = f(ws).mean(), f(ws).std() / np.sqrt(len(ws))
            b = 4 * np.pi * np.mean(qu * f(wu))
            sb = 4 * np.pi * np.std(qu * f(wu)) / np.sqrt(len(wu))
            assert abs(a - b) <= 4 * np.hypot(sa, sb)


def test_flat_layout_round_trip():
    p = G.init_params(5)
    flat = G.flatten(p)
    assert flat.size == G.N_PARAMS == native.GUIDE_PARAMS
    q = G.unflatten(flat)
    assert all(np.allclose(a[0], b[0], atol=1e-7) and np.allclose(a[1], b[1]) for a, b in zip(p, q))


def tiny_scene():
    return m.Scene.from_string(scenes.cornell(32, 32, 4, 5, 1))


def random_batch(n, seed):
    rng = np.random.default_rng(seed)
    feat = rng.uniform(0, 1, (n, 8)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.uniform(0.05, 3.0, n).astype(np.float32)
    return feat, d.astype(np.float32), w


@pytest.mark.gpu
def test_tensor_core_forward_matches_oracle(lib):
    guide = m.Guide(tiny_scene(), seed=11)
    params = G.unflatten(guide.params())
    # non-zero biases so that they are exercised too
    rng = np.random.default_rng(1)
    params = [(w, rng.normal(0, 0.1, b.shape)) for w, b in params]
    guide.set_params(G.flatten(params))
    params = G.unflatten(G.flatten(params))
    feat, _, _ = random_batch(1000, 2)
    got = guide.forward(feat)
    ref, _, _ = G.forward(params, feat.astype(np.float64), bf16_round=True)
    scale = np.abs(ref).max()
    err = np.abs(got - ref).max() / scale
    print(f"forward: max error {err:.3g} of the output scale {scale:.3g}")
    assert err < 2e-2
    assert np.corrcoef(got.ravel(), ref.ravel())[0, 1] > 0.9995


@pytest.mark.gpu
def test_tensor_core_forward_many_tiles(lib):
    """Enough rows that every CTA's two groups loop over several 128-row
    tiles (one CTA per SM), with a ragged last tile."""
    guide = m.Guide(tiny_scene(), seed=13)
    rng = np.random.default_rng(4)
    params = [(w, rng.normal(0, 0.1, b.shape)) for w, b in G.unflatten(guide.params())]
    guide.set_params(G.flatten(params))
    params = G.unflatten(G.flatten(params))
    n = 152 * 256 * 3 + 77
    feat, _, _ = random_batch(n, 5)
    got = guide.forward(feat)
    ref, _, _ = G.forward(params, feat.astype(np.float64), bf16_round=True)
    err = np.abs(got - ref).max(axis=1) / np.abs(ref).max()
    print(f"forward over {n} rows: max error {err.max():.3g} of the output scale")
    assert err.max() < 2e-2
    # rows are independent of their position: a row moved to another tile gives the same outputs
    again = guide.forward(feat[::-1].copy())[::-1]
    assert np.array_equal(again, got)


@pytest.mark.gpu
def test_training_gradients_match_oracle(lib):
    guide = m.Guide(tiny_scene(), seed=12)
    params = G.unflatten(guide.params())
    feat, d, w = random_batch(3000, 3)
    grad, loss = guide.gradients(feat, d, w)
    out, acts, zs = G.forward(params, feat.astype(np.float64), bf16_round=False)
    ref_loss, dout = G.loss_grad(out, d.astype(np.float64), w.astype(np.float64))
    ref = G.flatten(G.backward(params, acts, zs, dout)).astype(np.float64)
    rel = np.abs(grad - ref).max() / np.abs(ref).max()
    print(f"gradients: max error {rel:.3g} of the largest gradient; loss {loss:.6f} vs {ref_loss:.6f}")
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    assert rel < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("targets,fraction", [(native.GUIDE_DIRECT, 0.9), (native.GUIDE_DIRECT, 1.0),
                                              (native.GUIDE_ALL, 0.5)])
def test_guided_render_is_unbiased(lib, targets, fraction):
    """Plain and guided renders of the Cornell box converge to the same
    image, before and after training. With MUON_GUIDE_DIRECT even a light-hit
    ray drawn from the mixture alone (fraction 1) stays unbiased: light
    sampling covers every point of the light, and its MIS weights use the
    light-hit ray's density."""
    import torch

    scene = m.Scene.from_string(scenes.cornell(32, 32, 4096, 5, 1))
    plain = scene.render(pixel_samples=16384, seed=5)
    guide = m.Guide(scene, seed=3, wave_paths=1 << 20, batch=1 << 14, targets=targets, mixture_fraction=fraction)
    h, w = scene.height, scene.width
    s = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
    q = torch.zeros_like(s)
    c = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    for it in range(4):
        p = scene.params(pixel_samples=1024, seed=100 + it, sample_offset=1024 * it,
                         flags=native.RENDER_ACCUMULATE if it else 0)
        guide.render_device(p, s.data_ptr(), q.data_ptr(), c.data_ptr())
        guide.train(8)
    torch.cuda.synchronize()
    assert guide.samples() > 0
    gs, gq, gc = s.cpu().numpy(), q.cpu().numpy(), c.cpu().numpy()
    assert np.all(gc == 4096)
    mean_g = gs / gc[..., None]
    var_g = np.maximum(gq / gc[..., None] - mean_g ** 2, 0) / gc[..., None]
    mean_p, var_p = plain.mean(), plain.variance_of_mean()
    # Light paths are heavy-tailed: over 16 independent 65,536-spp renders of
    # this scene the image means spread 1.6x wider than the per-pixel sample
    # variances predict, so the image-mean bound allows for that factor.
    img_se = 1.6 * np.sqrt(var_g.sum() + var_p.sum()) / mean_g.size
    diff = mean_g.mean() - mean_p.mean()
    print(f"image mean guided {mean_g.mean():.5f} plain {mean_p.mean():.5f} ({diff / img_se:+.2f} se)")
    assert abs(diff) <= 4 * img_se
    z = (mean_g - mean_p) / np.sqrt(var_g + var_p + 1e-30)
    assert (np.abs(z) > 4).mean() <= 0.01


@pytest.mark.gpu
def test_trained_guide_lowers_variance(lib):
    """What the trained network gains: in a room lit only through a ceiling
    slit, light samples mostly hit the ceiling; after online training the
    guided light-hit ray finds the slit, and the per-sample variance at equal
    samples drops well below the plain tracer's, with the same mean."""
    import torch

    text = scenes.slit_room(64, 64, 16, 5, level=4, clutter=500, seed=2)
    scene = m.Scene.from_string(text)
    h, w = scene.height, scene.width

    def film():
        return [torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((h, w), dtype=torch.int32, device="cuda")]

    def stats(f):
        s, q, c = (x.cpu().numpy() for x in f)
        c = c[..., None].astype(np.float64)
        mean = s / c
        return mean, np.maximum(q / c - mean * mean, 0)

    plain = film()
    scene.render_device(scene.params(pixel_samples=2048, seed=21), *[x.data_ptr() for x in plain])
    guide = m.Guide(scene, seed=5, batch=1 << 16)
    warm = film()
    for it in range(24):
        guide.render_device(scene.params(pixel_samples=16, seed=200 + it, sample_offset=16 * it,
                                         flags=native.RENDER_ACCUMULATE if it else 0), *[x.data_ptr() for x in warm])
        guide.train(8)
    guided = film()
    guide.render_device(scene.params(pixel_samples=2048, seed=22), *[x.data_ptr() for x in guided])
    torch.cuda.synchronize()
    mp, vp = stats(plain)
    mg, vg = stats(guided)
    ratio = vg.mean() / vp.mean()
    se = np.sqrt((vp.sum() + vg.sum()) / 2048) / mp.size
    print(f"per-sample variance guided / plain {ratio:.3f}; image mean guided {mg.mean():.5f} "
          f"plain {mp.mean():.5f} ({(mg.mean() - mp.mean()) / se:+.2f} se)")
    assert ratio < 0.75
    assert abs(mg.mean() - mp.mean()) <= 4 * se


@pytest.mark.gpu
def test_guiding_scene_matches_reference_pixel_subset(lib):
    """The guiding benchmark's scene (slit room, 1024x1024, depth 10), plain
    and guided, z-tested per pixel against 256 seeded pixels that the
    reference build rendered at 65,536 spp each (pt65k_subset_slit_room.npz,
    make_fixtures.py). The plain render stands for the full-frame image the
    benchmark measures RMSE against; the guided one is the estimator the
    benchmark times, on the scene it is timed on."""
    import ast

    import torch
    from conftest import GOLDEN

    fx = np.load(f"{GOLDEN}/pt65k_subset_slit_room.npz")
    gen = ast.literal_eval(str(fx["generator"]))
    scene = m.Scene.from_string(scenes.slit_room(gen["width"], gen["height"], gen["spp"], gen["max_depth"],
                                                 seed=gen["seed"]))
    h, w = scene.height, scene.width
    px, py = fx["pixels"][:, 0], fx["pixels"][:, 1]
    n_ref = float(fx["spp"])
    mean_r = fx["sum"] / n_ref
    se2_r = np.maximum(fx["sum_sq"] / n_ref - mean_r ** 2, 0) * n_ref / (n_ref - 1) / n_ref

    def film():
        return [torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((h, w), dtype=torch.int32, device="cuda")]

    def check(f, label):
        s, q, c = (x.cpu().numpy()[py, px] for x in f)
        c = c[:, None].astype(np.float64)
        mean_g = s / c
        se2_g = np.maximum(q / c - mean_g ** 2, 0) * c / (c - 1) / c
        z = (mean_g - mean_r) / np.sqrt(se2_g + se2_r + 1e-30)
        frac = (np.abs(z) > 4).mean()
        se = 1.6 * np.sqrt(se2_g.sum() + se2_r.sum()) / mean_g.size
        diff = mean_g.mean() - mean_r.mean()
        print(f"{label}: |z|>4 on {frac * 100:.2f}% of pixel channels, subset mean gpu {mean_g.mean():.5f} "
              f"ref {mean_r.mean():.5f} ({diff / se:+.2f} se)")
        assert frac <= 0.02
        assert abs(diff) <= 4 * se

    plain = film()
    scene.render_device(scene.params(pixel_samples=1024, seed=31), *[x.data_ptr() for x in plain])
    check(plain, "plain")
    guide = m.Guide(scene, seed=3)
    warm = film()
    for it in range(2):
        guide.render_device(scene.params(pixel_samples=16, seed=40 + it, sample_offset=16 * it,
                                         flags=native.RENDER_ACCUMULATE if it else 0), *[x.data_ptr() for x in warm])
        guide.train(48)
    guided = film()
    guide.render_device(scene.params(pixel_samples=1024, seed=32), *[x.data_ptr() for x in guided])
    check(guided, "guided")


@pytest.mark.gpu
def test_gpu_mixture_sampler_and_density_match_oracle(lib):
    """The GPU's lobe sampling and density (the functions guided renders use,
    through muon_gpu_guide_sample): with the output layer's weights zeroed
    and its bias set to a chosen raw vector, every row's mixture is known.
    The densities the GPU returns match the oracle's at the same directions,
    and the sampled directions have the oracle density's moments."""
    guide = m.Guide(tiny_scene(), seed=21)
    rng = np.random.default_rng(9)
    for _ in range(2):
        raw = _strong_mixture(rng)
        params = G.unflatten(guide.params())
        params[-1] = (np.zeros_like(params[-1][0]), raw)
        guide.set_params(G.flatten(params))
        raw = raw.astype(np.float32).astype(np.float64)
        n = 200000
        feat = rng.uniform(0, 1, (n, 8)).astype(np.float32)
        dirs, pdf = guide.sample(feat, rng.random((n, 3)).astype(np.float32))
        assert np.allclose(np.linalg.norm(dirs, axis=1), 1.0, atol=1e-5)
        ref = G.mixture_pdf(np.broadcast_to(raw, (n, G.N_OUT)), dirs.astype(np.float64))
        rel = np.abs(pdf - ref) / ref
        print(f"density: median relative error {np.median(rel):.2e}, max {rel.max():.2e}")
        assert np.median(rel) < 1e-4 and rel.max() < 1e-2
        wu = _sphere_points(rng, 1_000_000)
        qu = G.mixture_pdf(np.broadcast_to(raw, (len(wu), G.N_OUT)), wu)
        d = dirs.astype(np.float64)
        for f in (lambda v: v[:, 0], lambda v: v[:, 1], lambda v: v[:, 2], lambda v: v[:, 0] * v[:, 1],
                  lambda v: v[:, 2] ** 2, lambda v: v[:, 0] * v[:, 2]):
            a, sa = f(d).mean(), f(d).std() / np.sqrt(n)
            b = 4 * np.pi * np.mean(qu * f(wu))
            sb = 4 * np.pi * np.std(qu * f(wu)) / np.sqrt(len(wu))
            assert abs(a - b) <= 4 * np.hypot(sa, sb)


@pytest.mark.gpu
def test_guided_training_is_reproducible(lib):
    """Light-sample training samples enter the pool at positions fixed by
    bounce, path and slot, batches are drawn with a seeded generator and the
    gradients are reduced in a fixed order: two guides trained the same way
    end with identical networks and render identical films."""
    import torch

    scene = m.Scene.from_string(scenes.slit_room(64, 64, 16, 5, level=3, clutter=200, seed=4))
    h, w = scene.height, scene.width

    def film():
        return [torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((h, w), dtype=torch.int32, device="cuda")]

    def run():
        guide = m.Guide(scene, seed=8, batch=1 << 14)
        warm = film()
        for it in range(3):
            guide.render_device(scene.params(pixel_samples=16, seed=60 + it, sample_offset=16 * it,
                                             flags=native.RENDER_ACCUMULATE if it else 0), *[x.data_ptr() for x in warm])
            guide.train(4)
        out = film()
        guide.render_device(scene.params(pixel_samples=32, seed=70), *[x.data_ptr() for x in out])
        torch.cuda.synchronize()
        params, samples = guide.params(), guide.samples()
        guide.close()
        return params, samples, [x.cpu().numpy() for x in out]

    p1, n1, f1 = run()
    p2, n2, f2 = run()
    assert n1 == n2 and n1 > 0
    assert np.array_equal(p1, p2)
    for a, b in zip(f1, f2):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_inference_timeout_status_reaches_the_host(lib):
    """The host side of a device wait that gave up: the status word an
    inference kernel sets is written here from the host (no device wait is
    made to run out). Guided renders and forward passes of that guide then
    return MUON_ERR_TIMEOUT, destroying it succeeds, and the scene renders
    with a fresh guide afterwards (the context stays usable)."""
    import torch

    scene = tiny_scene()
    h, w = scene.height, scene.width
    film = [torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, w), dtype=torch.int32, device="cuda")]
    ptrs = [x.data_ptr() for x in film]
    params = scene.params(pixel_samples=4, seed=3)
    guide = m.Guide(scene, seed=2, batch=1 << 12, pool_capacity=1 << 16)
    guide.render_device(params, *ptrs)
    guide.set_status(1)
    with pytest.raises(m.MuonError) as e:
        guide.render_device(params, *ptrs)
    assert e.value.code == 4 and "timed out" in str(e.value)
    feat, _, _ = random_batch(256, 9)
    with pytest.raises(m.MuonError) as e:
        guide.forward(feat)
    assert e.value.code == 4
    guide.close()
    fresh = m.Guide(scene, seed=2, batch=1 << 12, pool_capacity=1 << 16)
    fresh.render_device(params, *ptrs)
    torch.cuda.synchronize()
    assert np.isfinite(film[0].cpu().numpy()).all() and (film[2].cpu().numpy() == 4).all()
    fresh.close()
