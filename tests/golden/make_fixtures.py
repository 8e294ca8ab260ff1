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


if __name__ == "__main__":
    main()
