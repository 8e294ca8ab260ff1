"""Host parser semantics (muon/parser.cc:230-880) on small scene texts."""
import numpy as np
import pytest

import muon_gb300 as m
from muon_gb300 import native, scenes

CAM = "camera 0 0 5  0 0 0  0 1 0  45\n"


def parse(text):
    return m.parse_string(text)


def test_defaults(lib):
    p = parse(CAM)
    d, r = p.desc, p.params
    assert (d.width, d.height) == (150, 150)
    assert r.integrator == native.INTEGRATORS["raytracer"]
    assert (r.pixel_samples, r.light_samples, r.max_depth, r.min_depth) == (1, 1, 5, 0)
    assert r.next_event_estimation == 0 and r.importance_sampling == 0 and r.russian_roulette == 0
    assert p.gamma == 1.0 and p.output is None


def test_random_seed_falls_through_into_film_size(lib):
    # muon/parser.cc:267-286: the seed case has no break
    p = parse("random_seed 5 64 32\n" + CAM)
    assert (p.desc.width, p.desc.height) == (64, 32)
    p = parse("random_seed 5\n" + CAM)
    assert (p.desc.width, p.desc.height) == (150, 150)
    assert p.warnings == 1
    a = parse("random_seed 5\nintegrator pathtracer\n" + CAM).params.seed
    b = parse("random_seed 5\nintegrator pathtracer\n" + CAM).params.seed
    c = parse("random_seed 6\nintegrator pathtracer\n" + CAM).params.seed
    assert a == b != c
    # std::mt19937(5)'s first output
    assert a == 953453411


def test_camera_keeps_film_size_of_its_line(lib):
    p = parse("film_size 20 10\n" + CAM + "film_size 40 30\n")
    assert (p.desc.camera.width, p.desc.camera.height) == (20, 10)
    assert (p.desc.width, p.desc.height) == (40, 30)


def test_lambertian_builds_phong(lib):
    p = parse(CAM + "brdf lambertian\nsphere 0 0 0 1\nbrdf ggx\nsphere 0 0 0 1\n")
    mats = [p.desc.materials[p.desc.spheres[i].material] for i in range(2)]
    assert mats[0].brdf == 1 and mats[1].brdf == 2


def test_quad_light_adds_two_emissive_triangles(lib):
    p = parse(CAM + "ambient 0.3 0.3 0.3\nquad_light 1 2 3  1 0 0  0 0 2  5 6 7\n")
    d = p.desc
    assert d.num_triangles == 2 and d.num_lights == 1
    t0, t1 = d.triangles[0], d.triangles[1]
    v = lambda t: np.array([[t.v[k][j] for j in range(3)] for k in range(3)])
    va, vb, vc, vd = np.array([1, 2, 3.0]), np.array([2, 2, 3.0]), np.array([1, 2, 5.0]), np.array([2, 2, 5.0])
    assert np.array_equal(v(t0), [va, vc, vb]) and np.array_equal(v(t1), [vb, vc, vd])
    mat = d.materials[t0.material]
    assert list(mat.emission) == [5, 6, 7] and list(mat.ambient) == [0, 0, 0] and mat.brdf == 1
    assert t0.light == 0 and t0.transform == -1 and (t0.prim_id, t1.prim_id) == (0, 1)


def test_transform_stack_and_inverse(lib):
    p = parse(CAM + "push_transform\ntranslate 1 2 3\nrotate 0 1 0 90\nscale 2 2 2\nsphere 0 0 0 1\npop_transform\n"
              "sphere 0 0 0 1\n")
    d = p.desc
    s0, s1 = d.spheres[0], d.spheres[1]
    assert s1.transform == -1 and s0.transform >= 0
    t = d.transforms[s0.transform]
    M = np.array(t.object_to_world, dtype=np.float64).reshape(4, 4).T
    Minv = np.array(t.world_to_object, dtype=np.float64).reshape(4, 4).T
    T = np.eye(4); T[:3, 3] = [1, 2, 3]
    R = np.array([[0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0], [0, 0, 0, 1.0]])
    S = np.diag([2, 2, 2, 1.0])
    assert np.allclose(M, T @ R @ S, atol=1e-6)
    assert np.allclose(Minv @ M, np.eye(4), atol=1e-6)
    NT = np.array(t.normal_to_world, dtype=np.float64).reshape(4, 4).T
    assert np.allclose(NT, Minv.T, atol=0)


def test_vertex_normals_accumulate_and_normalise(lib):
    text = CAM + ("compute_vertex_normals on\nvertex 0 0 0\nvertex 1 0 0\nvertex 0 1 0\nvertex 0 0 1\n"
                  "tri 0 1 2\ntri 0 3 1\n")
    d = parse(text).desc
    n0 = np.array([d.triangles[0].n[0][j] for j in range(3)])
    assert np.allclose(n0, np.array([0, 1, 1]) / np.sqrt(2), atol=1e-7)
    assert d.triangles[0].smooth == 1


def test_bad_lines_are_skipped(lib):
    p = parse(CAM + "bogus 1 2\nsphere 1 2\ntri 0 1 99\nfilm_size x y\n")
    assert p.warnings == 4 and p.desc.num_spheres == 0 and p.desc.num_triangles == 0


@pytest.mark.parametrize("name", ["cornell", "sphere_field", "feature_mix"])
def test_synthetic_scenes_parse(lib, name):
    p = parse(scenes.WORKLOADS[name]())
    assert p.desc.num_triangles + p.desc.num_spheres > 0
    ids = sorted([p.desc.triangles[i].prim_id for i in range(p.desc.num_triangles)] +
                 [p.desc.spheres[i].prim_id for i in range(p.desc.num_spheres)])
    assert ids == list(range(len(ids)))


def test_benchmark_scenes_have_their_stated_sizes(lib):
    """The dense-mesh and guiding workloads as bench.py builds them contain
    the triangle counts its JSON line reports (a level-8 icosphere of
    1,310,720 triangles plus 10,000 clutter triangles, in the box or the
    slit room) and one quad light each."""
    import bench

    for name, make in [("dense_mesh", scenes.dense_mesh), ("guiding", scenes.slit_room)]:
        p = parse(make(64, 64, 1, 10))
        assert p.desc.num_triangles == bench.WORKLOADS[name]["triangles"], name
        assert p.desc.num_spheres == 0 and p.desc.num_lights == 1
    # the headline: 512 spheres, a ground quad and the 2x2 quad light (2 triangles each)
    p = parse(scenes.sphere_field(64, 64, 1, 8))
    assert p.desc.num_spheres == bench.WORKLOADS["sphere_field"]["spheres"] == 512
    assert p.desc.num_triangles == 4 and p.desc.num_lights == 1


def test_batch_scenes_follow_their_distribution(lib):
    """Every 8th scene of the 64-scene batch: triangle count within
    [1000, 500000] beyond the Cornell box's 36, a square resolution from
    {128, 256, 512, 1024}, spp in 4..64, max depth in 4..10 (what bench.py
    reports for the batch workload)."""
    import bench

    for i in range(0, bench.WORKLOADS["batch64"]["scenes"], 8):
        p = parse(scenes.batch_scene(i, bench.WORKLOADS["batch64"]["seed"]))
        d, r = p.desc, p.params
        assert 1000 <= d.num_triangles - 36 <= 500_000, (i, d.num_triangles)
        assert d.width == d.height and d.width in (128, 256, 512, 1024)
        assert 4 <= r.pixel_samples <= 64 and 4 <= r.max_depth <= 10


def test_cli_arguments(tmp_path):
    """The `muon` CLI (the reference's flags): usage, and the errors it
    reports before touching the GPU."""
    import os
    import subprocess

    cli = os.path.join(os.path.dirname(m.__file__), "lib", "muon")
    run = lambda *a: subprocess.run([cli, *a], capture_output=True, text=True)
    r = run("--help")
    assert r.returncode == 0 and "usage: muon --scene=FILE" in r.stdout
    r = run()
    assert r.returncode == 1 and "scene file is required" in r.stderr
    r = run("--bogus")
    assert r.returncode == 1 and "unknown flag --bogus" in r.stderr
    r = run("--scene=" + str(tmp_path / "missing.muon"))
    assert r.returncode == 1 and "parse failed" in r.stderr
    scene = tmp_path / "s.muon"
    scene.write_text(scenes.cornell(8, 8, 1, 2, 1))
    r = run("--scene=" + str(scene), "--acceleration=octree")
    assert r.returncode == 1 and "unknown value for acceleration" in r.stderr
    r = run("--scene=" + str(scene), "--partition_strategy=random")
    assert r.returncode == 1 and "unknown value for partition_strategy" in r.stderr
    r = run("--scene=" + str(scene), "--intersect_mode=approximate")
    assert r.returncode == 1 and "unknown value for intersect_mode" in r.stderr


def test_film_tonemap_and_files(tmp_path):
    """Film::WriteOutput's tone map (mean, pow(1/gamma), clamp to [0, 1], x255
    truncated) on a synthetic film, and the PNG and PPM files it writes
    decode to the same bytes."""
    from muon_gb300 import imageio

    rng = np.random.default_rng(3)
    h, w = 7, 9
    count = rng.integers(1, 50, (h, w)).astype(np.uint32)
    mean = rng.uniform(0, 1.3, (h, w, 3))
    film = m.FilmResult(mean * count[..., None], mean * mean * count[..., None], count)
    got = film.tonemap(1.0)
    want = (np.clip((film.sum / count[..., None]).astype(np.float32), 0, 1) * np.float32(255)).astype(np.uint8)
    assert np.array_equal(got, want)
    g22 = film.tonemap(2.2).astype(int)
    ref = np.clip(np.power((film.sum / count[..., None]).astype(np.float32), np.float32(1 / 2.2)), 0, 1)
    ref = (ref * np.float32(255)).astype(int)
    assert np.abs(g22 - ref).max() <= 1 and (g22 != ref).mean() < 0.01  # powf may differ from numpy by an ulp
    for name in ("f.png", "f.ppm"):
        path = str(tmp_path / name)
        film.write(path, 2.2)
        assert np.array_equal(imageio.read_image(path), film.tonemap(2.2))
