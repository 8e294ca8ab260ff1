"""Ray-level parity with the reference renderer on the GPU.

The golden fixtures hold the reference's own sample-0 camera rays and closest
hits (tests/golden/make_fixtures.py runs the reference build). In the EXACT
intersection mode the GPU repeats the reference's arithmetic, so wherever it
reports the same primitive the distance, normal and integrator outputs are
bit-identical. Primitive ids may differ only where two primitives are hit at
exactly the same distance (a ray through a shared edge), where the winner
depends on traversal order: the reference's own BVH and linear structures
disagree there too. Such pixels must stay below 0.5% and must be exact ties.
FAST and WATERTIGHT mode agree to the stated tolerances.
"""
import numpy as np
import pytest

import muon_gb300 as m
from conftest import GOLDEN
from muon_gb300 import native

SCENES = ["cornell", "sphere_field", "feature_mix", "dense_mesh"]


def load(name):
    return np.load(f"{GOLDEN}/hits_{name}.npz")


def ref_ids(fx):
    return np.where(fx["hit"] == 1, fx["prim_id"], -1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENES)
def test_exact_hits_are_bitwise_equal_to_reference(lib, name):
    fx = load(name)
    scene = m.Scene.from_string(str(fx["scene"]))
    rays = fx["rays"]
    dist, pid, pos, nrm = scene.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    rid = ref_ids(fx)
    agree = pid == rid
    tie = ~agree & (pid >= 0) & (rid >= 0) & (dist == fx["distance"])
    print(f"{name}: ids agree on {agree.mean() * 100:.4f}% of pixels, {int(tie.sum())} exact ties, "
          f"{int((~agree & ~tie).sum())} other")
    assert not (~agree & ~tie).any()
    assert tie.mean() <= 0.005
    both = agree & (rid >= 0)
    assert np.array_equal(dist[both], fx["distance"][both])
    assert np.array_equal(nrm[both], fx["normal"][both])


# (mode, relative distance tolerance, minimum id agreement)
LOOSE = [(native.ISECT_FAST, 5e-4, 0.995), (native.ISECT_WATERTIGHT, 5e-4, 0.995)]


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("mode,rtol,min_agree", LOOSE)
def test_fast_modes_agree_within_tolerance(lib, name, mode, rtol, min_agree):
    fx = load(name)
    scene = m.Scene.from_string(str(fx["scene"]))
    rays = fx["rays"]
    dist, pid, _, nrm = scene.intersect(rays[:, :3], rays[:, 3:], mode)
    rid = ref_ids(fx)
    agree = pid == rid
    print(f"{name} mode {mode}: ids agree on {agree.mean() * 100:.4f}%")
    assert agree.mean() >= min_agree
    both = agree & (rid >= 0)
    d_ref = fx["distance"][both]
    assert np.all(np.abs(dist[both] - d_ref) <= rtol * d_ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("mode", [native.ISECT_FAST, native.ISECT_WATERTIGHT, native.ISECT_EXACT])
def test_occlusion_matches_closest_hit(lib, name, mode):
    fx = load(name)
    scene = m.Scene.from_string(str(fx["scene"]))
    rays = fx["rays"]
    dist, pid, _, _ = scene.intersect(rays[:, :3], rays[:, 3:], mode)
    hit = pid >= 0
    far = np.where(hit, dist * 1.001, np.float32(1e30)).astype(np.float32)
    near = np.where(hit, dist * 0.999, np.float32(1e30)).astype(np.float32)
    assert np.array_equal(scene.occluded(rays[:, :3], rays[:, 3:], far, mode), hit)
    assert not scene.occluded(rays[:, :3], rays[:, 3:], near, mode)[hit].any()


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENES)
def test_occlusion_matches_the_reference_distances(lib, name):
    """Any hit (Structure::HasIntersection, muon/acceleration.cc:144-202)
    against the reference's own closest-hit distances: something lies within
    1.001 x the reference's distance exactly where the reference hit, and
    nothing lies within 0.999 x it."""
    fx = load(name)
    scene = m.Scene.from_string(str(fx["scene"]))
    rays = fx["rays"]
    hit = fx["hit"] == 1
    d = fx["distance"]
    far = np.where(hit, d * np.float32(1.001), np.float32(1e30)).astype(np.float32)
    near = np.where(hit, d * np.float32(0.999), np.float32(1e30)).astype(np.float32)
    assert np.array_equal(scene.occluded(rays[:, :3], rays[:, 3:], far, native.ISECT_EXACT), hit)
    assert not scene.occluded(rays[:, :3], rays[:, 3:], near, native.ISECT_EXACT)[hit].any()


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("integrator", ["normals", "albedo", "depth"])
def test_debug_integrators_are_bitwise_equal(lib, name, integrator):
    """NormalsTracer/AlbedoTracer/DepthTracer (muon/integration.cc:47-72) at
    sample 0: film values and 8-bit output equal the reference's."""
    fx = load(name)
    scene = m.Scene.from_string(str(fx["scene"]))
    film = scene.render(integrator=integrator, pixel_samples=1)
    assert np.all(film.count == 1)
    got = film.sum.reshape(-1, 3).astype(np.float32)
    hit = fx["hit"] == 1
    f = np.float32
    if integrator == "normals":
        ref = np.where(hit[:, None], fx["normal"] * f(0.5) + f(0.5), f(0))
    elif integrator == "albedo":
        ref = np.where(hit[:, None], fx["albedo"], f(0))
    else:
        ref = np.where(hit[:, None], f(1) / (f(1) + fx["distance"][:, None]), f(0))
        ref = np.repeat(ref, 3, axis=1)
    _, pid, _, _ = scene.intersect(fx["rays"][:, :3], fx["rays"][:, 3:], native.ISECT_EXACT)
    same = pid == ref_ids(fx)
    assert np.array_equal(got[same], ref[same].astype(np.float32))
    img = film.tonemap(1.0).reshape(-1, 3)
    ref8 = (np.minimum(np.maximum(ref.astype(np.float32), f(0)), f(1)) * f(255)).astype(np.uint8)
    differ = (img != ref8).any(axis=1)
    print(f"{name}/{integrator}: {int(differ.sum())} of {len(differ)} pixels differ in 8-bit output "
          f"({int((differ & ~same).sum())} of them at exact ties)")
    assert not (differ & same).any()


TINY = {
    "one_sphere": "film_size 16 16\ncamera 0 0 5  0 0 0  0 1 0  45\nsphere 0 0 0 1\n",
    "one_quad": ("film_size 16 16\ncamera 0 0 5  0 0 0  0 1 0  45\nstart_mesh\nvertex -1 -1 0\nvertex 1 -1 0\n"
                 "vertex 1 1 0\nvertex -1 1 0\ntri 0 1 2\ntri 0 2 3\nend_mesh\n"),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(TINY))
def test_scene_whose_bvh_root_is_a_leaf(lib, name):
    """With at most four primitives the whole BVH is one leaf; rays from
    outside its box must still find it."""
    from oracle import port

    text = TINY[name]
    rays = port.camera_rays(text)
    scene = m.Scene.from_string(text)
    dist, pid, _, _ = scene.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    d_ref, id_ref, _, _ = port.intersect(text, rays, precision=32, linear=True)
    assert (id_ref >= 0).sum() > 0
    assert np.array_equal(pid >= 0, id_ref >= 0)
    hit = id_ref >= 0
    assert np.array_equal(dist[hit], d_ref[hit].astype(np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENES)
def test_gpu_built_bvh_gives_the_same_hits(lib, name):
    """The device-built linear BVH (MUON_BUILDER_GPU_LBVH) holds every
    primitive exactly once: closest hits equal the reference's as with the
    host-built tree (ties aside), and any-hit queries agree with them."""
    fx = load(name)
    scene = m.Scene.from_string(str(fx["scene"]), builder="gpu")
    rays = fx["rays"]
    dist, pid, pos, nrm = scene.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    rid = ref_ids(fx)
    agree = pid == rid
    tie = ~agree & (pid >= 0) & (rid >= 0) & (dist == fx["distance"])
    assert not (~agree & ~tie).any()
    both = agree & (rid >= 0)
    assert np.array_equal(dist[both], fx["distance"][both])
    assert np.array_equal(nrm[both], fx["normal"][both])
    hit = pid >= 0
    far = np.where(hit, dist * 1.001, np.float32(1e30)).astype(np.float32)
    assert np.array_equal(scene.occluded(rays[:, :3], rays[:, 3:], far), hit)
    st_scene = m.Scene.from_string(str(fx["scene"]))
    a = scene.render(integrator="depth", pixel_samples=1)
    b = st_scene.render(integrator="depth", pixel_samples=1)
    same = agree | tie
    assert np.array_equal(a.sum.reshape(-1, 3)[same], b.sum.reshape(-1, 3)[same])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(TINY))
def test_gpu_built_bvh_of_a_tiny_scene(lib, name):
    text = TINY[name]
    from oracle import port

    rays = port.camera_rays(text)
    scene = m.Scene.from_string(text, builder="gpu")
    _, pid, _, _ = scene.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    _, id_ref, _, _ = port.intersect(text, rays, precision=32, linear=True)
    assert np.array_equal(pid >= 0, id_ref >= 0)
