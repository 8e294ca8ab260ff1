"""Batched rendering (muon_gpu_batch_*): several scenes in one wavefront.

A path's random numbers depend only on its scene's seed, pixel, sample and
bounce, and every scene keeps its own BVH, lights and settings inside the
merged image, so each film of a batched render must equal the film of the
same scene rendered alone with the same parameters, whatever the wave size,
traversal grid, scene order or mix of scenes in a wave. The batched shading
kernel is a separate compilation of the same code, and the compiler may fuse
a multiply and an add into one rounding in one and not the other, so values
may differ in the last bits: every pixel agrees to 1e-5 relative except a
rare path that such a last-bit difference sends another way (at most 0.5% of
pixels), sample counts agree exactly, and most pixels are bitwise equal.
"""
import numpy as np
import pytest

import muon_gb300 as m
from muon_gb300 import native, scenes


def small_batch():
    texts = [scenes.cornell(32, 32, 8, 5, 3),
             scenes.batch_scene(0, 7, max_tris=3000, resolutions=(16, 24, 40), spp_range=(2, 6), depth_range=(2, 6)),
             scenes.whitted(24, 24, 4, 5, 2, "pathtracer", "mis"),
             scenes.feature_mix(32, 32, 4, "pathtracer", "mis", 5),
             scenes.batch_scene(1, 7, max_tris=3000, resolutions=(16, 24, 40), spp_range=(2, 6), depth_range=(2, 6)),
             scenes.sphere_field(40, 24, 4, 6)]
    return [m.Scene.from_string(t) for t in texts]


def films_equal(a, b):
    if not np.array_equal(a.count, b.count):
        return False
    close = np.isclose(a.sum, b.sum, rtol=1e-5, atol=1e-12).all(axis=-1)
    same = (a.sum == b.sum).all(axis=-1)
    return close.mean() >= 0.995 and same.mean() >= 0.9


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [native.ISECT_EXACT, native.ISECT_FAST])
def test_batched_films_equal_single_scene_films(lib, mode):
    sc = small_batch()
    params = [s.params(intersect_mode=mode, flags=native.RENDER_STATS) for s in sc]
    single = [s.render(p) for s, p in zip(sc, params)]
    single_stats = [s.stats() for s in sc]
    batch = m.Batch(sc)
    got = batch.render(params)
    for i, (a, b) in enumerate(zip(got, single)):
        assert films_equal(a, b), f"scene {i} differs"
    total, per = batch.stats()
    assert [p["primary_rays"] for p in per] == [s["primary_rays"] for s in single_stats]
    assert total["secondary_rays"] == sum(s["secondary_rays"] for s in single_stats)
    assert total["shadow_rays"] == sum(s["shadow_rays"] for s in single_stats)
    assert all(p["done_ms"] > 0 for p in per)
    assert max(p["done_ms"] for p in per) <= total["render_ms"] + 1e-3
    batch.close()


@pytest.mark.gpu
def test_autotuned_batch_keeps_results(lib):
    sc = small_batch()
    params = [s.params() for s in sc]
    single = [s.render(p) for s, p in zip(sc, params)]
    batch = m.Batch(sc)
    tune = batch.autotune(params)
    assert tune["candidates"] >= 3
    assert tune["wave_paths"] >= 1 << 20 and 2 <= tune["traversal_blocks_per_sm"] <= 4
    got = batch.render(params)
    assert all(films_equal(a, b) for a, b in zip(got, single))
    batch.close()


@pytest.mark.gpu
def test_batch_rejects_what_it_cannot_render(lib):
    sc = small_batch()[:2]
    batch = m.Batch(sc)
    with pytest.raises(native.MuonError):
        batch.render([sc[0].params(intersect_mode=native.ISECT_FAST), sc[1].params(intersect_mode=native.ISECT_EXACT)])
    with pytest.raises(native.MuonError):
        batch.render([sc[0].params(integrator="normals"), sc[1].params()])
    with pytest.raises(native.MuonError):
        batch.render([sc[0].params(max_depth=-1), sc[1].params()])
    batch.close()
