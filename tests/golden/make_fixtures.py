"""Generates the committed golden fixtures from the reference renderer.

Runs the reference's own code (oracle/_ref/ref_driver, built from the
reference sources by oracle/Makefile) on the seeded synthetic scenes of
muon_gb300.scenes and stores small .npz files next to this script:

  hits_<name>.npz  sample-0 camera rays and the reference's closest hits
                   (linear structure: parse-order primitive ids; BVH: values)
  pt_<name>.npz    FP64 films of independent single-thread path-traced
                   renders (distinct seeds) for statistical parity tests
  img_<name>.npz   1-spp films of the deterministic ray tracer and analytic
                   direct integrators (FP32 values) and the ray counters
  pt65k_<name>.npz one single-thread render of 65,536 spp per path-traced
                   scene (seed 4242): a converged reference for per-pixel
                   z-tests, free of the correlation between runs that the
                   reference's unseeded first tile (muon/sampling.cc:41-46)
                   puts into pt_<name>.npz
  hits_dense_mesh_full.npz
                   65,536 seeded pixels of the benchmark's dense mesh itself
                   (1024x1024, 1,320,756 triangles): the reference BVH's
                   sample-0 closest hits, with parse-order ids recovered from
                   a key of the primitive hit (`hitkeys`), and the counters
                   of a 1-spp single-thread path-traced render of the frame;
                   the scene is regenerated from the stored generator call
  hits_batch13.npz, pt_batch13.npz
                   scene 13 of the 64-scene batch (356,235 triangles, 256x256,
                   depth 10): every pixel's sample-0 closest hit, and every
                   pixel traced at 1,024 spp by 8 processes on disjoint pixel
                   sets (`pixels` mode, so no run shares jitter positions)
  pt65k_subset_slit_room.npz
                   256 seeded pixels of the 1024x1024 guiding scene (slit
                   room, depth 10) at 65,536 spp each (8 processes of 8,192
                   with distinct seeds): the converged values that the GPU's
                   full-frame reference of the guiding benchmark, and guided
                   renders, are z-tested against; the scene is regenerated
                   from the stored generator arguments

Usage: python tests/golden/make_fixtures.py [--only NAME ...]
Requires the reference sources (to build oracle/_ref); the GPU machine only reads
the .npz files.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from muon_gb300 import scenes  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
HIT_DTYPE = np.dtype([("ray", "<f4", 6), ("hit", "<i4"), ("id", "<i4"), ("dist", "<f4"), ("pos", "<f4", 3),
                      ("normal", "<f4", 3), ("albedo", "<f4", 3)])

HIT_SCENES = {
    "cornell": lambda: scenes.cornell(128, 128, 1, 5, 1, "normals"),
    "sphere_field": lambda: scenes.sphere_field(128, 128, 1, 8).replace("integrator pathtracer", "integrator normals"),
    "feature_mix": lambda: scenes.feature_mix(128, 128, 1, "normals"),
    "dense_mesh": lambda: scenes.dense_mesh(128, 128, 1, 10, level=4, clutter=500).replace(
        "integrator pathtracer", "integrator normals"),
}

# deterministic integrators rendered at 1 spp (sample 0 = pixel centre)
IMG_SCENES = {
    "whitted_rt": lambda: scenes.whitted(128, 128, 1, 5, 1, "raytracer", "off"),
    "whitted_rt_nee": lambda: scenes.whitted(128, 128, 1, 4, 2, "raytracer", "on"),
    "whitted_analytic": lambda: scenes.whitted(128, 128, 1, 5, 3, "analyticdirect"),
    "cornell_analytic": lambda: scenes.cornell(128, 128, 1, 5, 1, "analyticdirect"),
}

# (scene text, runs, spp per run)
PT_SCENES = {
    "cornell": (lambda: scenes.cornell(32, 32, 64, 5, 1, "pathtracer"), 32, 1024),
    "feature_mix": (lambda: scenes.feature_mix(32, 32, 64, "pathtracer", "mis", 5), 32, 1024),
    "sphere_field": (lambda: scenes.sphere_field(32, 32, 64, 8), 32, 512),
    "cornell_nee_on": (lambda: scenes.cornell(32, 32, 64, 5, 1, "pathtracer", "on"), 32, 1024),
    "cornell_nee_off": (lambda: scenes.cornell(32, 32, 64, 5, 1, "pathtracer", "off"), 32, 1024),
    "dense_mesh": (lambda: scenes.dense_mesh(32, 32, 64, 10, level=3, clutter=200), 32, 512),
    # sampler and estimator options (muon/integration.cc:247-249, 313-321, 393-394, 503-562)
    "cornell_is_hemisphere": (lambda: scenes.cornell(32, 32, 64, 5, 1, "pathtracer").replace(
        "importance_sampling brdf", "importance_sampling hemisphere"), 32, 1024),
    "feature_mix_is_cosine": (lambda: scenes.feature_mix(32, 32, 64, "pathtracer", "mis", 5).replace(
        "importance_sampling brdf", "importance_sampling cosine"), 32, 1024),
    "cornell_rr_unbounded": (lambda: scenes.cornell(32, 32, 64, 5, 1, "pathtracer").replace(
        "russian_roulette off", "russian_roulette on").replace("max_depth 5", "max_depth -1"), 32, 1024),
    "cornell_stratified": (lambda: scenes.cornell(32, 32, 64, 5, 1, "pathtracer").replace(
        "russian_roulette off", "russian_roulette off\nlight_samples 4\nlight_stratify on"), 32, 512),
    "feature_mix_min_depth": (lambda: scenes.feature_mix(32, 32, 64, "pathtracer", "mis", 5).replace(
        "max_depth 5", "max_depth 5\nmin_depth 2"), 32, 1024),
}


def build_driver() -> None:
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "-s"], check=True)


def hits(name: str) -> None:
    text = HIT_SCENES[name]()
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "s.muon")
        open(sp, "w").write(text)
        recs = {}
        for mode in ("linear", "bvh"):
            out = os.path.join(td, mode + ".bin")
            subprocess.run([DRIVER, "hits", sp, out, mode], check=True)
            recs[mode] = np.fromfile(out, HIT_DTYPE)
    lin, bvh = recs["linear"], recs["bvh"]
    np.savez_compressed(os.path.join(HERE, f"hits_{name}.npz"), scene=np.array(text), rays=lin["ray"],
                        hit=lin["hit"].astype(np.int8), prim_id=lin["id"].astype(np.int32), distance=lin["dist"],
                        normal=lin["normal"], albedo=lin["albedo"], bvh_distance=bvh["dist"],
                        bvh_normal=bvh["normal"])
    print(f"hits_{name}: {len(lin)} rays, {int(lin['hit'].sum())} hits")


def _render(args) -> np.ndarray:
    text, spp, seed = args
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "s.muon")
        open(sp, "w").write(text)
        out = os.path.join(td, "f.bin")
        subprocess.run([DRIVER, "render", sp, out, str(spp), str(seed)], check=True)
        raw = open(out, "rb").read()
    w, h, n = np.frombuffer(raw, np.int32, 3)
    vals = np.frombuffer(raw, np.float64, 6 * w * h, offset=12)
    counters = np.frombuffer(raw, np.uint64, 4, offset=12 + 8 * 6 * w * h)
    return vals[:3 * w * h].reshape(h, w, 3), vals[3 * w * h:].reshape(h, w, 3), int(n), counters


def pt(name: str) -> None:
    make, runs, spp = PT_SCENES[name]
    text = make()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        res = list(ex.map(_render, [(text, spp, 1000 + r) for r in range(runs)]))
    sums = np.stack([r[0] for r in res])
    sqs = np.stack([r[1] for r in res])
    counters = np.stack([r[3] for r in res]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, f"pt_{name}.npz"), scene=np.array(text), sums=sums.astype(np.float64),
                        sum_sq=sqs.astype(np.float64), spp=np.int32(spp), counters=counters)
    print(f"pt_{name}: {runs} runs x {spp} spp, mean {sums.sum(0).mean() / (runs * spp):.4f}")


def img(name: str) -> None:
    text = IMG_SCENES[name]()
    s, _, n, counters = _render((text, 1, 1))
    np.savez_compressed(os.path.join(HERE, f"img_{name}.npz"), scene=np.array(text), film=s.astype(np.float32),
                        counters=counters.astype(np.int64))
    print(f"img_{name}: mean {s.mean():.5f}, counters {counters.tolist()}")


PT65K_SPP = 65536


def _pt65k(name: str) -> str:
    make, _, _ = PT_SCENES[name]
    text = make()
    s, q, n, counters = _render((text, PT65K_SPP, 4242))
    np.savez_compressed(os.path.join(HERE, f"pt65k_{name}.npz"), scene=np.array(text), sum=s.astype(np.float64),
                        sum_sq=q.astype(np.float64), spp=np.int32(PT65K_SPP), counters=counters.astype(np.int64))
    return f"pt65k_{name}: {PT65K_SPP} spp, mean {np.nanmean(s) / PT65K_SPP:.6f}"


def pt65k(names: list[str]) -> None:
    """One long render per scene, the scenes on parallel host threads."""
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for line in ex.map(_pt65k, names):
            print(line, flush=True)


SUBSET = {"width": 1024, "height": 1024, "spp": 16, "max_depth": 10, "seed": 1, "pixels": 256, "pixel_seed": 7,
          "processes": 8, "spp_per_process": 8192}


def _subset_run(args) -> tuple[np.ndarray, np.ndarray]:
    scene_path, pix_path, seed = args
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.run([DRIVER, "pixels", scene_path, pix_path, out, str(SUBSET["spp_per_process"]), str(seed)],
                       check=True)
        raw = open(out, "rb").read()
    n = int(np.frombuffer(raw, np.int32, 1)[0])
    vals = np.frombuffer(raw, np.float64, offset=8)
    return vals[:3 * n].reshape(n, 3), vals[3 * n:6 * n].reshape(n, 3)


def pt65k_subset() -> None:
    c = SUBSET
    text = scenes.slit_room(c["width"], c["height"], c["spp"], c["max_depth"], seed=c["seed"])
    rng = np.random.default_rng(c["pixel_seed"])
    flat = rng.choice(c["width"] * c["height"], size=c["pixels"], replace=False)
    pix = np.stack([flat % c["width"], flat // c["width"]], 1).astype(np.int32)
    with tempfile.TemporaryDirectory() as td:
        sp, pp = os.path.join(td, "s.muon"), os.path.join(td, "p.bin")
        open(sp, "w").write(text)
        pix.tofile(pp)
        with ThreadPoolExecutor(max_workers=c["processes"]) as ex:
            res = list(ex.map(_subset_run, [(sp, pp, 2000 + i) for i in range(c["processes"])]))
    sums = sum(r[0] for r in res)
    sqs = sum(r[1] for r in res)
    spp = c["processes"] * c["spp_per_process"]
    np.savez_compressed(os.path.join(HERE, "pt65k_subset_slit_room.npz"), pixels=pix, sum=sums, sum_sq=sqs,
                        spp=np.int32(spp), generator=np.array(str(c)))
    print(f"pt65k_subset_slit_room: {len(pix)} px x {spp} spp, mean {np.nanmean(sums) / spp:.6f}")


HIT_KEY_DTYPE = np.dtype([("ray", "<f4", 6), ("hit", "<i4"), ("kind", "<i4"), ("dist", "<f4"), ("pos", "<f4", 3),
                          ("normal", "<f4", 3), ("albedo", "<f4", 3), ("bounds", "<f4", 6), ("face", "<f4", 3),
                          ("xf", "<f4", 16)])


def _prim_keys(text: str) -> tuple[dict, dict]:
    """Key (object bounds, unnormalised face normal, object-to-world matrix;
    as `hitkeys` writes it) -> parse-order ids, from the repository's parser;
    and per triangle id its world-space vertices (FP64), for telling apart
    triangles with equal keys (the two halves of a planar quad)."""
    import ctypes as C

    import muon_gb300 as m

    parsed = m.parse_string(text)
    d = parsed.desc
    xf = np.frombuffer(C.string_at(d.transforms, d.num_transforms * 192), np.float32).reshape(-1, 48)[:, :16] \
        if d.num_transforms else np.zeros((0, 16), np.float32)
    ident = np.eye(4, dtype=np.float32).reshape(16)
    tdt = np.dtype([("v", "<f4", (3, 3)), ("n", "<f4", (3, 3)), ("transform", "<i4"), ("material", "<i4"),
                    ("light", "<i4"), ("smooth", "<i4"), ("prim_id", "<i4"), ("pad", "<i4")])
    tris = np.frombuffer(C.string_at(d.triangles, d.num_triangles * tdt.itemsize), tdt)
    v = tris["v"]
    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]  # float32, as the reference's Tri constructor
    face = np.stack([e1[:, 1] * e2[:, 2] - e2[:, 1] * e1[:, 2], e1[:, 2] * e2[:, 0] - e2[:, 2] * e1[:, 0],
                     e1[:, 0] * e2[:, 1] - e2[:, 0] * e1[:, 1]], 1).astype(np.float32)
    lo, hi = v.min(axis=1), v.max(axis=1)
    mats = np.where(tris["transform"][:, None] >= 0, xf[np.maximum(tris["transform"], 0)] if len(xf) else ident,
                    ident)
    keys = np.concatenate([lo, hi, face, mats], 1).astype(np.float32)
    out: dict = {}
    for k, pid in zip(map(bytes, keys.view(np.uint8).reshape(len(keys), -1)), tris["prim_id"]):
        out.setdefault(k, []).append(int(pid))
    # world-space vertices of the triangles that share a key with another
    shared = {pid for ids in out.values() if len(ids) > 1 for pid in ids}
    row = {int(p): i for i, p in enumerate(tris["prim_id"]) if int(p) in shared}
    world = {}
    for pid, i in row.items():
        mat = mats[i].astype(np.float64).reshape(4, 4).T  # column-major -> rows
        vh = np.concatenate([v[i].astype(np.float64), np.ones((3, 1))], 1)
        world[pid] = (vh @ mat.T)[:, :3]
    sdt = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("transform", "<i4"), ("material", "<i4"),
                    ("prim_id", "<i4"), ("pad", "<i4")])
    sph = np.frombuffer(C.string_at(d.spheres, d.num_spheres * sdt.itemsize), sdt)
    for s in sph:
        c, r = s["center"], np.float32(s["radius"])
        mat = xf[s["transform"]] if s["transform"] >= 0 else ident
        k = np.concatenate([c - r, c + r, np.zeros(3, np.float32), mat]).astype(np.float32)
        out.setdefault(bytes(k.view(np.uint8)), []).append(int(s["prim_id"]))
    parsed.close()
    return out, world


def _outside(tri: np.ndarray, p: np.ndarray) -> float:
    """How far p lies outside a triangle's barycentric range (0 inside)."""
    a, b, c = tri
    n = np.cross(b - a, c - a)
    nn = n @ n
    w = [np.cross(c - b, p - b) @ n / nn, np.cross(a - c, p - c) @ n / nn, np.cross(b - a, p - a) @ n / nn]
    return float(max(0.0, -min(w)))


def _hitkeys(text: str, pix: np.ndarray) -> np.ndarray:
    with tempfile.TemporaryDirectory() as td:
        sp, pp, out = os.path.join(td, "s.muon"), os.path.join(td, "p.bin"), os.path.join(td, "o.bin")
        open(sp, "w").write(text)
        pix.astype(np.int32).tofile(pp)
        subprocess.run([DRIVER, "hitkeys", sp, pp, out], check=True)
        return np.fromfile(out, HIT_KEY_DTYPE)


def _keyed_hit_fixture(path: str, text: str, pix: np.ndarray, extra: dict) -> None:
    import hashlib
    import zlib

    rec = _hitkeys(text, pix)
    keys, world = _prim_keys(text)
    kbytes = np.concatenate([rec["bounds"], rec["face"], rec["xf"]], 1).astype(np.float32)
    ids = np.full(len(rec), -1, np.int32)
    ambiguous = unmatched = 0
    for i in np.nonzero(rec["hit"] == 1)[0]:
        cand = keys.get(bytes(kbytes[i].view(np.uint8)), [])
        if len(cand) == 1:
            ids[i] = cand[0]
            continue
        if not cand:
            ids[i] = -3  # no primitive with this key (not expected)
            unmatched += 1
            continue
        # equal keys: the candidate whose world triangle holds the hit point
        p = rec["pos"][i].astype(np.float64)
        out = sorted((_outside(world[c], p), c) for c in cand)
        if out[0][0] < 1e-7 and out[1][0] > 1e-4:
            ids[i] = out[0][1]
        else:
            ids[i] = -3  # on (or near) the shared edge: no unique answer
            ambiguous += 1
    np.savez_compressed(path, pixels=pix.astype(np.int32), ray_crc=np.uint32(zlib.crc32(rec["ray"].tobytes())),
                        hit=rec["hit"].astype(np.int8), prim_id=ids, distance=rec["dist"], normal=rec["normal"],
                        albedo=rec["albedo"], scene_sha256=np.array(hashlib.sha256(text.encode()).hexdigest()),
                        **extra)
    print(f"{os.path.basename(path)}: {len(rec)} pixels, {int(rec['hit'].sum())} hits, {ambiguous} on shared "
          f"edges, {unmatched} unmatched keys")


FULL_DENSE = {"width": 1024, "height": 1024, "spp": 1, "max_depth": 10, "pixels": 65536, "pixel_seed": 11}


def hits_dense_mesh_full() -> None:
    c = FULL_DENSE
    text = scenes.dense_mesh(c["width"], c["height"], 256, c["max_depth"])
    rng = np.random.default_rng(c["pixel_seed"])
    flat = np.sort(rng.choice(c["width"] * c["height"], size=c["pixels"], replace=False))
    pix = np.stack([flat % c["width"], flat // c["width"]], 1).astype(np.int32)
    # counted rays of the full frame at 1 spp (one thread, seed 1)
    _, _, _, counters = _render((text, 1, 1))
    _keyed_hit_fixture(os.path.join(HERE, "hits_dense_mesh_full.npz"), text, pix,
                       {"generator": np.array("scenes.dense_mesh(1024, 1024, 256, 10)"),
                        "counters_1spp": counters.astype(np.int64)})


BATCH13 = {"index": 13, "seed": 1, "spp": 1024, "processes": 8}


def batch13() -> None:
    c = BATCH13
    text = scenes.batch_scene(c["index"], c["seed"])
    import re

    w, h = map(int, re.search(r"film_size (\d+) (\d+)", text).groups())
    ys, xs = np.mgrid[0:h, 0:w]
    pix = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    _keyed_hit_fixture(os.path.join(HERE, "hits_batch13.npz"), text, pix,
                       {"generator": np.array(f"scenes.batch_scene({c['index']}, {c['seed']})")})
    # converged values: disjoint pixel sets per process, each pixel traced spp times
    parts = np.array_split(np.arange(len(pix)), c["processes"])
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "s.muon")
        open(sp, "w").write(text)
        jobs = []
        for i, idx in enumerate(parts):
            pp = os.path.join(td, f"p{i}.bin")
            pix[idx].tofile(pp)
            jobs.append((sp, pp, 3000 + i, c["spp"]))
        with ThreadPoolExecutor(max_workers=c["processes"]) as ex:
            res = list(ex.map(_pixels_run, jobs))
    s = np.zeros((len(pix), 3))
    q = np.zeros((len(pix), 3))
    for idx, (a, b) in zip(parts, res):
        s[idx], q[idx] = a, b
    np.savez_compressed(os.path.join(HERE, "pt_batch13.npz"), sum=s.reshape(h, w, 3), sum_sq=q.reshape(h, w, 3),
                        spp=np.int32(c["spp"]), generator=np.array(f"scenes.batch_scene({c['index']}, {c['seed']})"))
    print(f"pt_batch13: {w}x{h} x {c['spp']} spp, mean {np.nanmean(s) / c['spp']:.6f}")


def _pixels_run(args) -> tuple[np.ndarray, np.ndarray]:
    scene_path, pix_path, seed, spp = args
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.run([DRIVER, "pixels", scene_path, pix_path, out, str(spp), str(seed)], check=True)
        raw = open(out, "rb").read()
    n = int(np.frombuffer(raw, np.int32, 1)[0])
    vals = np.frombuffer(raw, np.float64, offset=8)
    return vals[:3 * n].reshape(n, 3), vals[3 * n:6 * n].reshape(n, 3)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    a = ap.parse_args()
    build_driver()
    for name in HIT_SCENES:
        if not a.only or name in a.only:
            hits(name)
    for name in PT_SCENES:
        if not a.only or ("pt_" + name) in a.only:
            pt(name)
    for name in IMG_SCENES:
        if not a.only or ("img_" + name) in a.only:
            img(name)
    pt65k([name for name in PT_SCENES if not a.only or ("pt65k_" + name) in a.only])
    if not a.only or "pt65k_subset_slit_room" in a.only:
        pt65k_subset()
    if not a.only or "hits_dense_mesh_full" in a.only:
        hits_dense_mesh_full()
    if not a.only or "batch13" in a.only:
        batch13()


if __name__ == "__main__":
    main()
