"""The device binned-SAH builder (MUON_BUILDER_GPU_SAH) against the host one.

With this builder the triangles' records are computed on the device too
(scene_records.cu, the host builder's arithmetic), so the comparisons below
also pin the device records: boxes, hit distances in the object-space exact
mode, and normals (smooth ones included) must be the host's bits.

It takes the host builder's split decisions with the same float operations,
so the two trees must have the same nodes: the same multiset of (padded
child box, child box, leaf contents) rows, the same partition of primitives
into leaves, and the same statistics. Only node numbering and the order of
primitives inside a leaf may differ. Hits then equal the host tree's (and so
the reference's) except exact ties between primitives of one leaf. Checked
on the parity fixture scenes, the full benchmark scenes, tiny scenes, other
leaf sizes, and a scene whose centroids all coincide (halves by position,
where only validity and hits are compared).
"""
import numpy as np
import pytest

import muon_gb300 as m
from conftest import GOLDEN
from muon_gb300 import native, scenes

FIXTURE_SCENES = ["cornell", "sphere_field", "feature_mix", "dense_mesh"]

TINY = {
    "one_triangle": ("film_size 8 8\ncamera 0 0 5  0 0 0  0 1 0  45\nstart_mesh\nvertex -1 -1 0\nvertex 1 -1 0\n"
                     "vertex 0 1 0\ntri 0 1 2\nend_mesh\n"),
    "one_sphere": "film_size 8 8\ncamera 0 0 5  0 0 0  0 1 0  45\nsphere 0 0 0 1\n",
    "three_spheres": ("film_size 8 8\ncamera 0 0 9  0 0 0  0 1 0  45\nsphere -2 0 0 1\nsphere 0 0 0 1\n"
                      "sphere 2 0 0 1\n"),
    "six_spheres": "film_size 8 8\ncamera 0 0 9  0 0 0  0 1 0  45\n" +
                   "".join(f"sphere {x} {y} 0 0.4\n" for x in (-2, 0, 2) for y in (-1, 1)),
}


def _leaf_keys(prim, last):
    """Per primitive id, the smallest primitive id of its leaf; per slot, the
    leaf's key."""
    ends = np.flatnonzero(last)
    starts = np.concatenate([[0], ends[:-1] + 1])
    leaf_of_slot = np.repeat(np.arange(len(ends)), ends - starts + 1)
    leaf_min = np.minimum.reduceat(prim, starts)
    slot_key = leaf_min[leaf_of_slot]
    by_prim = np.full(prim.max() + 1, -1, dtype=np.int64)
    by_prim[prim] = slot_key
    return by_prim, slot_key, starts


def _canonical(nodes, prim, last, slot_order=True):
    """Rows of (each child's box as bits and leaf key, -1 for an interior
    child), sorted: equal for two trees with the same nodes whatever their
    numbering. Without slot_order the two children of a node are sorted too."""
    bits = nodes.view(np.uint32).astype(np.int64)
    links = nodes.view(np.int32)[:, 12:14]
    _, slot_key, _ = _leaf_keys(prim, last)
    kid = np.where(links < 0, slot_key[np.where(links < 0, ~links, 0)], -1).astype(np.int64)
    c0 = np.concatenate([bits[:, [0, 1, 2, 3, 8, 9]], kid[:, :1]], axis=1)
    c1 = np.concatenate([bits[:, [4, 5, 6, 7, 10, 11]], kid[:, 1:]], axis=1)
    if not slot_order:
        swap = np.lexsort(np.concatenate([c0, c1], axis=0).T[::-1]).argsort()
        first = swap[:len(c0)] < swap[len(c0):]
        c0, c1 = np.where(first[:, None], c0, c1), np.where(first[:, None], c1, c0)
    rows = np.concatenate([c0, c1], axis=1)
    return rows[np.lexsort(rows.T[::-1])]


def _check_valid(info, nodes, prim, last, n_prims, max_leaf):
    """Every primitive in exactly one leaf, leaves no larger than max_leaf,
    every node reached once from the root."""
    assert len(prim) == n_prims and len(np.unique(prim)) == n_prims
    _, _, starts = _leaf_keys(prim, last)
    sizes = np.diff(np.concatenate([starts, [len(prim)]]))
    assert sizes.max() <= max(max_leaf, 1) or info["nodes"] == 1
    links = nodes.view(np.int32)[:, 12:14]
    seen = np.zeros(len(nodes), dtype=np.int64)
    leaf_seen = np.zeros(len(prim), dtype=np.int64)
    stack = [0]
    while stack:
        i = stack.pop()
        seen[i] += 1
        for link in links[i]:
            if link >= 0:
                stack.append(int(link))
            else:
                leaf_seen[~link] += 1
    assert (seen == 1).all()
    if info["nodes"] > 1:
        assert (leaf_seen[starts] == 1).all()


def _same_tree(text, slot_order=True, **kw):
    host = m.Scene.from_string(text, builder="host", **kw)
    dev = m.Scene.from_string(text, builder="gpu_sah", **kw)
    hi, hn, hp, hl = host.bvh()
    di, dn, dp, dl = dev.bvh()
    for k in ("nodes", "slots", "leaves", "max_depth", "max_leaf"):
        assert hi[k] == di[k], (k, hi[k], di[k])
    assert np.array_equal(_leaf_keys(hp, hl)[0], _leaf_keys(dp, dl)[0])
    a, b = _canonical(hn, hp, hl, slot_order), _canonical(dn, dp, dl, slot_order)
    print(f"{len(a)} nodes, {int((a != b).any(axis=1).sum())} canonical rows differ")
    assert np.array_equal(a, b)
    return host, dev


def _hits_agree(host, dev, rays):
    d0, p0, _, n0 = host.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    d1, p1, _, n1 = dev.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    assert np.array_equal(p0 >= 0, p1 >= 0)
    assert np.array_equal(d0, d1)
    same = p0 == p1
    # a different primitive only at an exact tie (the distances are equal):
    # two triangles of a quad in one leaf, tested in another order
    print(f"ids equal on {same.mean() * 100:.4f}% of {len(same)} rays")
    assert same.mean() >= 0.995
    assert np.array_equal(n0[same], n1[same])


@pytest.mark.gpu
@pytest.mark.parametrize("name", FIXTURE_SCENES)
def test_device_sah_tree_equals_the_host_tree(lib, name):
    fx = np.load(f"{GOLDEN}/hits_{name}.npz")
    host, dev = _same_tree(str(fx["scene"]))
    _hits_agree(host, dev, fx["rays"])
    # and against the reference's hits, as the host tree is checked
    rid = np.where(fx["hit"] == 1, fx["prim_id"], -1)
    dist, pid, _, _ = dev.intersect(fx["rays"][:, :3], fx["rays"][:, 3:], native.ISECT_EXACT)
    tie = (pid != rid) & (pid >= 0) & (rid >= 0) & (dist == fx["distance"])
    assert not ((pid != rid) & ~tie).any()
    host.close()
    dev.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(TINY))
def test_device_sah_tree_of_a_tiny_scene(lib, name):
    host, dev = _same_tree(TINY[name])
    info, nodes, prim, last = dev.bvh()
    _check_valid(info, nodes, prim, last, info["slots"], 4)


@pytest.mark.gpu
@pytest.mark.parametrize("max_leaf", [1, 2, 8])
def test_device_sah_tree_with_other_leaf_sizes(lib, max_leaf):
    """With one primitive per leaf, two primitives whose centroids coincide
    are split by the median rule, which puts them in either slot (the host's
    nth_element orders equal keys its own way): there the children of a node
    are compared as a set."""
    fx = np.load(f"{GOLDEN}/hits_dense_mesh.npz")
    host, dev = _same_tree(str(fx["scene"]), slot_order=max_leaf > 1, max_leaf_size=max_leaf)
    info, nodes, prim, last = dev.bvh()
    _check_valid(info, nodes, prim, last, info["slots"], max_leaf)
    _hits_agree(host, dev, fx["rays"])


@pytest.mark.gpu
def test_device_sah_tree_of_coincident_centroids(lib):
    """4,100 copies of one triangle and a few others: nodes whose centroids
    all coincide are halved by position (the host's median split orders equal
    keys its own way), so only validity and hit distances are compared."""
    tri = "tri 0 1 2\n" * 4100
    text = ("film_size 64 64\ncamera 0 0 5  0 0 0  0 1 0  45\nstart_mesh\nvertex -1 -1 0\nvertex 1 -1 0\n"
            "vertex 0 1 0\n" + tri + "end_mesh\nsphere 2 2 -1 0.5\nsphere -2 -2 -1 0.5\n")
    host = m.Scene.from_string(text, builder="host")
    dev = m.Scene.from_string(text, builder="gpu_sah")
    info, nodes, prim, last = dev.bvh()
    _check_valid(info, nodes, prim, last, 4102, 4)
    assert info["leaves"] == host.bvh()[0]["leaves"]
    from oracle import port

    rays = port.camera_rays(text)
    d0, p0, _, _ = host.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    d1, p1, _, _ = dev.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    assert (p0 >= 0).sum() > 0
    assert np.array_equal(p0 >= 0, p1 >= 0)
    assert np.array_equal(d0, d1)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["dense_mesh_full", "batch13"])
def test_device_sah_tree_of_the_benchmark_scenes(lib, which):
    """The headline dense mesh (1,320,756 triangles) and batch scene 13: the
    same tree as the host's, and the same hits on the fixture pixels."""
    fx = np.load(f"{GOLDEN}/hits_{which}.npz")
    text = scenes.dense_mesh(1024, 1024, 256, 10) if which == "dense_mesh_full" else scenes.batch_scene(13, 1)
    host, dev = _same_tree(text)
    from oracle import port

    pix = fx["pixels"]
    rays = port.camera_rays(text)[pix[:, 1] * host.width + pix[:, 0]]
    _hits_agree(host, dev, rays)
    host.close()
    dev.close()


def _smooth_scene():
    """A smooth-shaded (compute_vertex_normals) wavy grid under a rotation
    and scale, a second copy without smoothing, spheres and a quad light."""
    import math

    k = 40
    verts = [f"vertex {x / k * 2 - 1:.5f} {y / k * 2 - 1:.5f} {0.15 * math.sin(5 * x / k) * math.cos(4 * y / k):.5f}"
             for y in range(k + 1) for x in range(k + 1)]
    tris = []
    for y in range(k):
        for x in range(k):
            a = y * (k + 1) + x
            tris += [f"tri {a} {a + 1} {a + k + 2}", f"tri {a} {a + k + 2} {a + k + 1}"]
    mesh = "start_mesh\n" + "\n".join(verts + tris) + "\nend_mesh\n"
    return ("camera 0 0 6  0 0 0  0 1 0  45\nfilm_size 96 96\n"
            "quad_light 2 2 2  -1 3 1  0 0.5 0  0.5 0 0\n"
            "push_transform\nrotate 1 0.3 0.2 35\nscale 1.2 0.9 1.1\ncompute_vertex_normals on\n" + mesh +
            "pop_transform\ncompute_vertex_normals off\npush_transform\ntranslate 0 0 -1.5\n" + mesh +
            "pop_transform\nsphere 1.5 1.5 0 0.4\nsphere -1.5 -1.2 0.5 0.3\n")


@pytest.mark.gpu
def test_device_records_of_a_smooth_transformed_scene(lib):
    text = _smooth_scene()
    parsed = m.parse_string(text)
    assert any(parsed.desc.triangles[i].smooth for i in range(parsed.desc.num_triangles))
    host, dev = _same_tree(text)
    from oracle import port

    rays = port.camera_rays(text)
    _hits_agree(host, dev, rays)
    # the normals film interpolates the smooth vertex normals
    a = host.render(integrator="normals", pixel_samples=1)
    b = dev.render(integrator="normals", pixel_samples=1)
    _, p0, _, _ = host.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    _, p1, _, _ = dev.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
    same = p0 == p1
    assert np.array_equal(a.sum.reshape(-1, 3)[same], b.sum.reshape(-1, 3)[same])


@pytest.mark.gpu
def test_device_build_of_degenerate_and_sphere_only_scenes(lib):
    """Only never-hit (zero-area) triangles: no tree and no hits, as with the
    host build; only spheres: no triangle records, the same tree."""
    from oracle import port

    flat = ("film_size 16 16\ncamera 0 0 5  0 0 0  0 1 0  45\nstart_mesh\nvertex 0 0 0\nvertex 1 0 0\nvertex 2 0 0\n"
            "tri 0 1 2\ntri 1 2 0\nend_mesh\n")
    for builder in ("host", "gpu_sah"):
        sc = m.Scene.from_string(flat, builder=builder)
        info = sc.bvh()[0]
        assert info["nodes"] == 0 and info["slots"] == 0
        rays = port.camera_rays(flat)
        _, pid, _, _ = sc.intersect(rays[:, :3], rays[:, 3:], native.ISECT_EXACT)
        assert (pid < 0).all()
        film = sc.render(integrator="depth", pixel_samples=1)
        assert not film.sum.any()
    spheres = "film_size 16 16\ncamera 0 0 9  0 0 0  0 1 0  45\n" + "".join(
        f"sphere {x * 0.7 - 3} {(x * 37 % 11) * 0.5 - 2.5} {(x * 13 % 7) * 0.3} 0.3\n" for x in range(300))
    host, dev = _same_tree(spheres)
    _hits_agree(host, dev, port.camera_rays(spheres))
