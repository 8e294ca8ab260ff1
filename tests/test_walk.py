"""The host walk of the flattened BVH (muon_walk_rays, muon_gpu_probe_traversal).

The walk counts traversal work (box tests and primitive tests, what the
reference's TraceStats counts, muon/stats.h:11-44) on the very arrays the GPU
traverses, in the GPU's visiting order; the benchmark's algorithmic bytes
come from it. On the CPU: it finds the reference build's closest hits on the
hit fixtures (so it walks the same BVH to the same answers), and its any-hit
answer agrees with its closest hit. On the GPU: a render's host-walked counts
equal the traversal kernels' own counters.
"""
import numpy as np
import pytest

import muon_gb300 as m
from conftest import GOLDEN
from muon_gb300 import native, scenes

SCENES = ["cornell", "sphere_field", "feature_mix", "dense_mesh"]


@pytest.mark.parametrize("name", SCENES)
def test_host_walk_finds_the_reference_closest_hits(lib, name):
    fx = np.load(f"{GOLDEN}/hits_{name}.npz")
    parsed = m.parse_string(str(fx["scene"]))
    rays = fx["rays"]
    ids, cnt = m.walk_rays(parsed, rays[:, :3], rays[:, 3:], intersect_mode=native.ISECT_EXACT)
    rid = np.where(fx["hit"] == 1, fx["prim_id"], -1)
    agree = ids == rid
    # a disagreement is a tie: both hit something, at the reference's distance
    # (checked on the GPU, bitwise, by the hit tests); few of them
    assert ((ids >= 0) == (rid >= 0)).all()
    assert (~agree).mean() <= 0.005
    assert cnt["rays"] == len(rays) and cnt["hits"] == int((rid >= 0).sum())
    # every walk tests the root's two boxes; hits need at least one primitive test
    assert cnt["box_tests"] >= 2 * len(rays) and cnt["prim_tests"] >= cnt["hits"]
    print(f"{name}: {cnt['box_tests'] / len(rays):.1f} box tests, {cnt['prim_tests'] / len(rays):.2f} "
          f"primitive tests per ray; ids agree on {agree.mean() * 100:.3f}%")


@pytest.mark.parametrize("name", ["cornell", "dense_mesh"])
def test_host_any_hit_agrees_with_closest_hit(lib, name):
    fx = np.load(f"{GOLDEN}/hits_{name}.npz")
    parsed = m.parse_string(str(fx["scene"]))
    rays = fx["rays"]
    ids, _ = m.walk_rays(parsed, rays[:, :3], rays[:, 3:], intersect_mode=native.ISECT_EXACT)
    dist = fx["distance"]
    hit = ids >= 0
    beyond = np.where(hit, dist * np.float32(1.001), np.float32(1e30)).astype(np.float32)
    short = np.where(hit, dist * np.float32(0.999), np.float32(1e30)).astype(np.float32)
    occ_far, c_far = m.walk_rays(parsed, rays[:, :3], rays[:, 3:], beyond, any_hit=True)
    occ_near, c_near = m.walk_rays(parsed, rays[:, :3], rays[:, 3:], short, any_hit=True)
    assert ((occ_far >= 0) == hit).all()
    # nothing lies in front of the closest hit (a miss has no limit and stays a miss)
    assert not (occ_near[hit] >= 0).any()
    assert c_far["hits"] == int(hit.sum())


def test_host_walk_rejects_watertight_mode(lib):
    parsed = m.parse_string(scenes.cornell(8, 8, 1, 5, 1))
    with pytest.raises(m.MuonError):
        m.walk_rays(parsed, np.zeros((1, 3)), np.array([[0, 0, -1.0]]), intersect_mode=native.ISECT_WATERTIGHT)


@pytest.mark.gpu
@pytest.mark.parametrize("name,kwargs", [("cornell", {}), ("sphere_field", {}), ("dense_mesh", {"level": 4})])
def test_probe_counts_match_the_gpu_counters(lib, name, kwargs):
    """Every queued ray of a small render walked on the host, in the ordered
    visiting sequence: the traversal kernels count the same work plus what
    their speculative descent adds (a lane that postpones a leaf descends
    further before the leaf's hit shortens the ray), never less, and at most
    a fifth more (13% on the sphere field, whose lanes often reach leaves
    together)."""
    if name == "cornell":
        text = scenes.cornell(32, 32, 4, 5, 1)
    elif name == "sphere_field":
        text = scenes.sphere_field(32, 32, 4, 6)
    else:
        text = scenes.dense_mesh(32, 32, 4, 6, clutter=500, seed=2, **kwargs)
    scene = m.Scene.from_string(text)
    p = scene.params(intersect_mode=native.ISECT_EXACT, seed=5)
    pr = scene.probe_traversal(p, rays_per_queue=1 << 20)
    st = scene.stats()
    assert pr["extend_rays"] == st["extend_rays"] and pr["occlude_rays"] == st["occlude_rays"]
    assert pr["extend_walked"]["rays"] == st["extend_rays"]  # every ray sampled
    for host, gpu in [(pr["extend_box_tests"], st["extend_box_tests"]),
                      (pr["extend_prim_tests"], st["extend_prim_tests"]),
                      (pr["occlude_box_tests"], st["occlude_box_tests"]),
                      (pr["occlude_prim_tests"], st["occlude_prim_tests"])]:
        assert 0.8 * gpu <= host <= gpu * 1.001 + 2
    print(f"{name}: extend {st['extend_box_tests']} box / {st['extend_prim_tests']} prim tests, host "
          f"{pr['extend_box_tests']:.0f} / {pr['extend_prim_tests']:.0f}; occlude {st['occlude_box_tests']} / "
          f"{st['occlude_prim_tests']}, host {pr['occlude_box_tests']:.0f} / {pr['occlude_prim_tests']:.0f}")


@pytest.mark.gpu
def test_probe_sample_estimates_the_whole_render(lib):
    """A sample of each queue, scaled by its length, estimates the whole
    render's traversal work to within a few percent."""
    scene = m.Scene.from_string(scenes.sphere_field(128, 128, 8, 6))
    p = scene.params(intersect_mode=native.ISECT_EXACT, seed=9)
    pr = scene.probe_traversal(p, rays_per_queue=2048)
    st = scene.stats()
    assert pr["extend_walked"]["rays"] < st["extend_rays"]
    for host, gpu in [(pr["extend_box_tests"], st["extend_box_tests"]),
                      (pr["occlude_box_tests"], st["occlude_box_tests"])]:
        assert 0.8 < host / gpu < 1.05


@pytest.mark.gpu
def test_read_bandwidth_ceilings_are_ordered(lib):
    """L1 above L2 above DRAM, and DRAM near the copy bandwidth class of an
    HBM3e part (not a fixed number: a sanity ordering)."""
    l1 = m.measure_read_bandwidth(0, 32 << 10, 500)
    l2 = m.measure_read_bandwidth(1, 24 << 20, 200)
    dram = m.measure_read_bandwidth(2, 4 << 30, 3)
    print(f"read GB/s: L1 {l1:.0f}, L2 {l2:.0f}, DRAM {dram:.0f}")
    assert l1 > l2 > dram > 1000


def test_scene_validation_reports_the_first_bad_triangle(lib):
    """Triangle indices are checked on all host threads; the error names the
    first bad triangle in input order, as a serial check would."""
    parsed = m.parse_string(scenes.dense_mesh(16, 16, 1, 2, level=6, clutter=2000, seed=3))
    d = parsed.desc
    assert d.num_triangles > 1 << 16
    tris = d.triangles
    k1, k2 = d.num_triangles // 3, 2 * d.num_triangles // 3
    saved = (tris[k1].material, tris[k2].transform)
    tris[k2].transform = d.num_transforms + 5  # later: a missing transform
    tris[k1].material = d.num_materials       # first: a missing material
    with pytest.raises(m.MuonError, match="missing material"):
        m.walk_rays(parsed, np.zeros((1, 3)), np.array([[0, 0, -1.0]]))
    tris[k1].material = saved[0]
    with pytest.raises(m.MuonError, match="missing transform"):
        m.walk_rays(parsed, np.zeros((1, 3)), np.array([[0, 0, -1.0]]))
    tris[k2].transform = saved[1]
    tris[k2].prim_id = d.num_triangles + d.num_spheres
    with pytest.raises(m.MuonError, match="primitive id out of range"):
        m.walk_rays(parsed, np.zeros((1, 3)), np.array([[0, 0, -1.0]]))
