"""Benchmark: path-traced Mrays/s on the random sphere field.

Workload (one step = one full frame): 512 seeded spheres (centres U[-10,10]^3,
radii U[0.2,1]), Lambertian / Phong / GGX materials, ground quad, one 2x2
quad light of emission 10; 512x512 pixels, 64 samples per pixel, max depth 8,
next-event estimation with MIS, BRDF importance sampling, FP32 shading, FP64
film. Synthetic and seeded (muon_gb300.scenes.sphere_field).

Metric: Mrays/s counted as the reference counts rays (primary + secondary,
the MIS-sampled ray included; shadow rays excluded, muon/integration.cc:34-38,
483), over device time with the scene resident and the film in device memory.
`e2e` is the same metric through the public API with host buffers: scene
upload (BVH build + copy) and the host film read-back inside every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload sphere_field|dense_mesh]

`--workload dense_mesh` measures the traversal-bound scene instead: a
1,310,720-triangle displaced icosphere (GGX roughness 0.15) and 10,000 small
clutter triangles in the Cornell box, 1024x1024, 256 spp, max depth 10, NEE
with MIS (muon_gb300.scenes.dense_mesh).

With N > 1 (torchrun), every rank renders its own replica of the frame with a
distinct seed (weak scaling; the FP64 films of replicas merge by addition).
`--impl reference` times the reference algorithm on the host cores: the
reference build when it runs on this machine, else the oracle's restatement.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the headline workload
    "sphere_field": {"workload": "sphere_field", "spheres": 512, "width": 512, "height": 512, "spp": 64,
                     "max_depth": 8, "nee": "mis", "importance_sampling": "brdf", "seed": 1},
    # traversal-bound: 1,310,720-triangle displaced icosphere (level 8) + 10k clutter triangles in the Cornell box
    "dense_mesh": {"workload": "dense_mesh", "triangles": 1320756, "width": 1024, "height": 1024, "spp": 256,
                   "max_depth": 10, "nee": "mis", "importance_sampling": "brdf", "seed": 1},
    # learned path guiding: time to RMSE 1e-2 against a converged plain render, guided vs plain
    "guiding": {"workload": "slit_room", "triangles": 1310720 + 10000 + 14 + 2, "width": 1024, "height": 1024,
                "max_depth": 10, "nee": "mis", "importance_sampling": "brdf", "seed": 1, "target_rmse": 1e-2,
                "reference_spp": 8192, "pass_spp": 16, "train_steps_per_pass": 128, "train_passes": 2,
                "batch": 1 << 18, "guide_targets": "direct", "mixture_fraction": 0.95, "guided_bounces": 4},
    # 64 seeded scenes of uneven size in one batched wavefront
    "batch64": {"workload": "batch64", "scenes": 64, "triangles": "log-uniform 1k-500k per scene",
                "resolutions": [128, 256, 512, 1024], "spp": "uniform 4-64", "max_depth": "uniform 4-10",
                "nee": "mis", "importance_sampling": "brdf", "seed": 1},
}
WORKLOAD = dict(WORKLOADS["sphere_field"])
METRIC = "Mrays/s"


def scene_text() -> str:
    from muon_gb300 import scenes

    w = WORKLOAD
    if w["workload"] == "dense_mesh":
        return scenes.dense_mesh(w["width"], w["height"], w["spp"], w["max_depth"], seed=w["seed"])
    return scenes.sphere_field(w["width"], w["height"], w["spp"], w["max_depth"], w["spheres"], w["seed"], w["nee"])


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples: list[list[str]] = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 2 + k and s[2 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def algorithmic_bytes(st: dict, slots: int) -> dict:
    """Bytes each kernel class must move per frame by its algorithm.

    Traversal (extend / occlude): 64 B per BVH node visited (two child boxes
    and links; box tests count 2 per node), 64 B per primitive record tested,
    plus the ray/hit records: extend reads a 32 B ray and writes an 8 B hit;
    occlude reads a 4 B queue entry, a 16 B origin and a 16 B direction.
    Shade, per shaded path: reads ray 32 + hit 8 + radiance 16 + throughput 16,
    writes radiance 16 + link 4 (counted in fold) + slots 48*S (clear, value,
    direction); per continuation +48 (ray 32, throughput 16); per shadow ray +4.
    Fold, per shaded path: reads radiance 16 + slots 16*S + link 4, writes 16.
    """
    ext = 32 * st["extend_box_tests"] + 64 * st["extend_prim_tests"] + 40 * st["extend_rays"]
    occ = 32 * st["occlude_box_tests"] + 64 * st["occlude_prim_tests"] + 36 * st["occlude_rays"]
    shaded = st["extend_rays"]
    cont = max(0, st["extend_rays"] - st["primary_rays"])
    shade = shaded * (88 + 48 * slots) + 48 * cont + 4 * st["shadow_rays"]
    fold = shaded * (16 + 16 * slots + 4 + 16)
    return {"extend": ext, "occlude": occ, "shade": shade, "fold": fold}


def batch_texts() -> list[str]:
    from muon_gb300 import scenes

    return [scenes.batch_scene(i, WORKLOAD["seed"]) for i in range(WORKLOAD["scenes"])]


def run_batch(args) -> None:
    """One step = one batched render of all 64 scenes (muon_gpu_batch_render_device)."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    from muon_gb300 import build as native_build

    native_build.build()
    import muon_gb300 as m
    from muon_gb300 import native, replicas

    texts = batch_texts()
    parsed = [m.parse_string(t) for t in texts]
    sc = [m.Scene(p, builder=args.builder) for p in parsed]
    batch = m.Batch(sc)
    params = [s.params(intersect_mode=native.ISECT_EXACT, seed=1000 * rank + i) for i, s in enumerate(sc)]
    t_tune = time.perf_counter()
    tune = batch.autotune(params)
    t_tune = time.perf_counter() - t_tune
    films = [(torch.zeros((s.height, s.width, 3), dtype=torch.float64, device="cuda"),
              torch.zeros((s.height, s.width, 3), dtype=torch.float64, device="cuda"),
              torch.zeros((s.height, s.width), dtype=torch.int32, device="cuda")) for s in sc]
    ptrs = [[f[k].data_ptr() for f in films] for k in range(3)]
    render = lambda: batch.render_device(params, *ptrs)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        render()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    times, counted, lat = [], 0, []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            render()
            total, per = batch.stats()
            times.append(total["render_ms"])
            counted += total["primary_rays"] + total["secondary_rays"]
            lat += [p["done_ms"] for p in per]
            launches = total["kernel_launches"]
    dev_ms = sum(times)
    dev_ms, counted = replicas.reduce_step(dev_ms, counted, device="cuda")
    value = counted / (dev_ms * 1e3)
    # end to end: scene uploads (BVH builds), batch merge, render, host films back
    e2e_steps = 2
    h2d = sum(p.desc.num_triangles * 80 + p.desc.num_spheres * 32 + p.desc.num_materials * 56 +
              p.desc.num_lights * 52 + p.desc.num_transforms * 192 for p in parsed)
    d2h = sum(s.width * s.height * (3 * 8 * 2 + 4) for s in sc)
    t0 = time.perf_counter()
    e2e_counted = 0
    for _ in range(e2e_steps):
        scs = [m.Scene(p, builder=args.builder) for p in parsed]
        b2 = m.Batch(scs)
        b2.render(params)
        tot, _ = b2.stats()
        e2e_counted += tot["primary_rays"] + tot["secondary_rays"]
        b2.close()
        for s in scs:
            s.close()
    e2e_value = e2e_counted / (time.perf_counter() - t0) / 1e6
    if rank != 0:
        return
    lat_sorted = sorted(lat)
    pct = lambda q: lat_sorted[min(len(lat_sorted) - 1, int(q * len(lat_sorted)))]
    cpu = None
    if world == 1:
        threads = os.cpu_count() or 1
        rates = [reference_rate(texts[i], 1, threads) for i in range(4)]
        rays = sum(r[0] * r[1] for r in rates)
        secs = sum(r[1] for r in rates)
        cpu = {"value": round(rays / secs, 3), "unit": METRIC, "cores": threads, "kind": rates[0][2],
               "sample": f"scenes 0-3 of the batch at 1 spp, {secs:.1f} s on {threads} threads"}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (64 seeded scenes)",
        "config": dict(WORKLOAD, parallelism=f"replicas{world}", intersect_mode="exact", bvh_builder=args.builder,
                       total_triangles=int(sum(p.desc.num_triangles for p in parsed)),
                       paths_per_step=int(total["paths"]),
                       l2="flushed between steps (256 MiB write)"),
        "latency_ms": {"p50": round(pct(0.50), 3), "p99": round(pct(0.99), 3), "max": round(lat_sorted[-1], 3),
                       "note": "per scene: batch start to its film complete"},
        "autotune": dict(tune, seconds=round(t_tune, 2)),
        "e2e": {"value": round(e2e_value, 2), "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "note": "64 scene uploads (BVH builds) + batch merge + render + host films back per step"},
        "gpu_launches": int(launches) * args.steps,
        "clocks": clocks.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def run_guiding(args) -> None:
    """Time to reach RMSE 1e-2 against a converged plain render of the slit
    room: the plain GPU tracer and the guided one (training time included),
    both rendering progressive passes of `pass_spp` samples; device time with
    CUDA events, the RMSE evaluations between passes excluded."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    from muon_gb300 import build as native_build

    native_build.build()
    import muon_gb300 as m
    from muon_gb300 import native, scenes

    w = WORKLOAD
    text = scenes.slit_room(w["width"], w["height"], w["pass_spp"], w["max_depth"], seed=w["seed"])
    scene = m.Scene.from_string(text)
    H, W = scene.height, scene.width
    stream = torch.cuda.ExternalStream(scene.stream())

    def film():
        return (torch.zeros((H, W, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((H, W, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((H, W), dtype=torch.int32, device="cuda"))

    ptr = lambda f: [x.data_ptr() for x in f]
    # converged reference, plain tracer, in passes of at most 256 spp
    ref = film()
    t0 = time.perf_counter()
    done = 0
    while done < w["reference_spp"]:
        n = min(256, w["reference_spp"] - done)
        scene.render_device(scene.params(pixel_samples=n, seed=7777, sample_offset=done,
                                         flags=native.RENDER_ACCUMULATE if done else 0), *ptr(ref))
        done += n
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t0
    ref_img = ref[0] / ref[2][..., None].double()

    def rmse(f):
        img = f[0] / f[2].clamp(min=1)[..., None].double()
        return float(torch.sqrt(((img - ref_img) ** 2).mean()))

    def progressive(render_pass, train=None, max_passes=4096):
        f = film()
        dev_ms, spp, passes, counted = 0.0, 0, 0, 0
        trace = []
        while passes < max_passes:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream.wait_stream(torch.cuda.current_stream())
            e0.record(stream)
            counted += render_pass(f, spp)
            if train is not None:
                train()
            e1.record(stream)
            torch.cuda.synchronize()
            dev_ms += e0.elapsed_time(e1)
            spp += w["pass_spp"]
            passes += 1
            err = rmse(f)
            trace.append((spp, round(dev_ms, 2), round(err, 5)))
            if err <= w["target_rmse"]:
                break
        return dev_ms, spp, err, counted, trace

    # passes launch kernel by kernel: a graph would be captured again for
    # every pass (its sample offset changes)
    def plain_pass(f, spp):
        scene.render_device(scene.params(pixel_samples=w["pass_spp"], seed=11, sample_offset=spp,
                                         flags=native.RENDER_NO_GRAPH | (native.RENDER_ACCUMULATE if spp else 0)),
                            *ptr(f))
        st = scene.stats()
        return st["primary_rays"] + st["secondary_rays"]

    guide = m.Guide(scene, seed=w["seed"], batch=w["batch"], mixture_fraction=w["mixture_fraction"],
                    record_bounces=w["guided_bounces"],
                    targets=native.GUIDE_DIRECT if w["guide_targets"] == "direct" else native.GUIDE_ALL)

    def guided_pass(f, spp):
        guide.render_device(scene.params(pixel_samples=w["pass_spp"], seed=12, sample_offset=spp,
                                         flags=native.RENDER_NO_GRAPH | (native.RENDER_ACCUMULATE if spp else 0)),
                            *ptr(f))
        st = scene.stats()
        return st["primary_rays"] + st["secondary_rays"]

    passes_trained = [0]

    def train():
        # online training during the first passes, then the network is frozen
        if passes_trained[0] < w["train_passes"]:
            guide.train(w["train_steps_per_pass"])
            passes_trained[0] += 1

    plain_ms, plain_spp, plain_err, plain_rays, plain_trace = progressive(plain_pass)
    guided_ms, guided_spp, guided_err, guided_rays, guided_trace = progressive(guided_pass, train=train)
    if rank != 0:
        return
    line = {
        "metric": "time-to-RMSE 1e-2 (guided / plain)", "value": round(guided_ms / plain_ms, 4), "unit": "ratio",
        "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": False, "scaling": "none", "vs_baseline": None,
        "dtype": "f32 (bf16 network)", "data": "synthetic (seeded slit room)",
        "config": dict(WORKLOAD, reference_seconds=round(ref_s, 2)),
        "plain": {"ms": round(plain_ms, 1), "spp": plain_spp, "rmse": round(plain_err, 5),
                  "mrays_per_s": round(plain_rays / (plain_ms * 1e3), 1)},
        "guided": {"ms": round(guided_ms, 1), "spp": guided_spp, "rmse": round(guided_err, 5),
                   "mrays_per_s": round(guided_rays / (guided_ms * 1e3), 1), "samples": guide.samples()},
        "trace_plain": plain_trace[-8:], "trace_guided": guided_trace[-8:],
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import numpy as np
    import torch

    if WORKLOAD["workload"] == "batch64":
        return run_batch(args)
    if WORKLOAD["workload"] == "slit_room":
        return run_guiding(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)

    from muon_gb300 import build as native_build

    native_build.build()
    import muon_gb300 as m
    from muon_gb300 import native, replicas

    text = scene_text()
    scene = m.Scene.from_string(text, builder=args.builder)
    seed = 1000 + rank
    # Every kernel is timed with CUDA events inside the frame's graph; the
    # frame time below includes that cost.
    params = scene.params(seed=seed, intersect_mode=native.ISECT_EXACT, flags=native.RENDER_TIMING)
    h, w = scene.height, scene.width
    d_sum = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
    d_sq = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
    d_cnt = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    render = lambda p: scene.render_device(p, d_sum.data_ptr(), d_sq.data_ptr(), d_cnt.data_ptr())

    # traversal work per frame (stats kernels), outside the timed region
    cal = scene.params(seed=seed, intersect_mode=native.ISECT_EXACT, flags=native.RENDER_STATS)
    render(cal)
    cal_stats = scene.stats()
    slots = 2  # one area light sample + the MIS ray per path vertex

    stream = torch.cuda.ExternalStream(scene.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # 256 MiB > 129 MB L2
    for _ in range(args.warmup):
        render(params)
    torch.cuda.synchronize()

    per_step, st_steps = [], []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            stream.wait_stream(torch.cuda.current_stream())
            ev[k][0].record(stream)
            render(params)
            ev[k][1].record(stream)
            st_steps.append(scene.stats())
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        wall = time.perf_counter() - t0
    per_step = [a.elapsed_time(b) for a, b in ev]
    dev_ms = sum(per_step)
    counted = sum(s["primary_rays"] + s["secondary_rays"] for s in st_steps)
    launches = sum(s["kernel_launches"] for s in st_steps)

    dev_ms_max, counted_all = replicas.reduce_step(dev_ms, counted, device="cuda")
    value = counted_all / (dev_ms_max * 1e3)

    # end to end through the public API with host buffers
    e2e_steps = max(2, min(args.steps, 5))
    parsed = m.parse_string(text)
    desc_bytes = (parsed.desc.num_triangles * 80 + parsed.desc.num_spheres * 32 + parsed.desc.num_materials * 56 +
                  parsed.desc.num_lights * 52 + parsed.desc.num_transforms * 192)
    film_bytes = h * w * (3 * 8 * 2 + 4)
    # the step's film comes back into pinned host memory, reused across steps
    host_film = m.FilmResult(torch.zeros((h, w, 3), dtype=torch.float64).pin_memory().numpy(),
                             torch.zeros((h, w, 3), dtype=torch.float64).pin_memory().numpy(),
                             torch.zeros((h, w), dtype=torch.int32).pin_memory().numpy().view(np.uint32))
    m.Scene(parsed, builder=args.builder).render(params, out=host_film)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_counted = 0
    for _ in range(e2e_steps):
        sc = m.Scene(parsed, builder=args.builder)
        sc.render(params, out=host_film)
        st = sc.stats()
        e2e_counted += st["primary_rays"] + st["secondary_rays"]
        sc.close()
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_counted / e2e_s / 1e6

    if rank != 0:
        return

    # roofline of the dominant kernel class
    last = st_steps[-1]
    alg = algorithmic_bytes(cal_stats, slots)
    times = {"extend": last["extend_ms"], "occlude": last["occlude_ms"], "shade": last["shade_ms"],
             "fold": last["fold_ms"]}
    dom = max(times, key=times.get)
    n_launch = {"extend": last["extend_launches"], "occlude": last["occlude_launches"],
                "shade": last["extend_launches"], "fold": last["extend_launches"]}[dom]
    per_launch_bytes = alg[dom] / max(1, n_launch)
    per_launch_ms = times[dom] / max(1, n_launch)
    pk = peaks()
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get(WORKLOAD["workload"], {}).get(dom)

    cpu = cpu_baseline(text) if world == 1 else None
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms_max / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": f"synthetic (seeded {WORKLOAD['workload'].replace('_', ' ')})",
        "config": dict(WORKLOAD, parallelism=f"replicas{world}", intersect_mode="exact", bvh_builder=args.builder,
                       l2="flushed between steps (256 MiB write)", counted_rays_per_step=counted // args.steps),
        "e2e": {"value": round(e2e_value, 2), "unit": METRIC, "h2d_bytes_per_step": int(desc_bytes),
                "d2h_bytes_per_step": int(film_bytes),
                "note": "scene upload (BVH build + copy) + render + film read-back into pinned host memory per step"},
        "gpu_launches": int(launches),
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": traffic,
                     "peak_source": pk["source"], "per_launch_bytes": int(per_launch_bytes),
                     "per_launch_ms": round(per_launch_ms, 4), "kernel_ms_per_step": {k: round(v, 3) for k, v in times.items()}},
        "clocks": clocks.summary(),
        "wall_s": round(wall, 3),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def _reference_binary() -> str | None:
    """The reference build (oracle/_ref) when it exists and runs here."""
    exe = os.path.join(ROOT, "oracle", "_ref", "muon_ref")
    if not os.path.exists(exe):
        return None
    try:
        r = subprocess.run([exe, "--help"], capture_output=True, timeout=10)
        return exe if r.returncode in (0, 1) else None
    except Exception:
        return None


def reference_rate(text: str, spp: int, threads: int) -> tuple[float, float, str]:
    """Counted Mrays/s of the reference algorithm on `threads` host threads for
    the workload at `spp` samples per pixel; returns (rate, seconds, kind)."""
    from oracle import port

    t0 = time.perf_counter()
    f = port.render(text, spp=spp, seed=1, threads=threads)
    el = time.perf_counter() - t0
    counted = f.counters["primary"] + f.counters["secondary"]
    return counted / el / 1e6, el, "port"


def cpu_baseline(text: str) -> dict:
    threads = os.cpu_count() or 1
    w, h = WORKLOAD["width"], WORKLOAD["height"]
    rate1, el1, kind = reference_rate(text, 1, threads)
    spp = max(1, min(WORKLOAD["spp"], int(10.0 / max(el1, 1e-3))))
    rate, el, kind = reference_rate(text, spp, threads)
    return {"value": round(rate, 3), "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"full {w}x{h} frame at {spp} spp (of {WORKLOAD['spp']}), {el:.1f} s on {threads} threads"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from oracle import build as oracle_build

    oracle_build.build()
    threads = os.cpu_count() or 1
    if WORKLOAD["workload"] == "batch64":
        # a bounded sample of the batch: its first scene at 1 spp per step
        text = batch_texts()[0]
        spp = 1
        sample = "scene 0 of the batch at 1 spp per step"
    else:
        text = scene_text()
        rate1, el1, kind = reference_rate(text, 1, threads)
        spp = max(1, min(WORKLOAD["spp"], int(5.0 / max(el1, 1e-3))))
        sample = f"full {WORKLOAD['width']}x{WORKLOAD['height']} frame at {spp} spp (of {WORKLOAD['spp']}) per step"
    for _ in range(args.warmup):
        reference_rate(text, 1, threads)
    rates, times = [], []
    for _ in range(args.steps):
        r, el, kind = reference_rate(text, spp, threads)
        rates.append(r)
        times.append(el)
    value = sum(rates) / len(rates)
    line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic (seeded {WORKLOAD['workload'].replace('_', ' ')})",
            "config": dict(WORKLOAD, parallelism=f"host threads {threads}"),
            "cpu_baseline": {"value": round(value, 3), "unit": METRIC, "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="sphere_field")
    ap.add_argument("--builder", choices=["host", "gpu"], default="host",
                    help="BVH builder: binned SAH on the host, or the linear BVH built on the GPU")
    ap.add_argument("--guide-targets", choices=["direct", "all"], default=None,
                    help="guiding workload: what the network learns (default: direct light)")
    ap.add_argument("--mixture-fraction", type=float, default=None,
                    help="guiding workload: probability that a guided ray samples the mixture")
    a = ap.parse_args()
    WORKLOAD.clear()
    WORKLOAD.update(WORKLOADS[a.workload])
    if a.workload == "guiding":
        if a.guide_targets:
            WORKLOAD["guide_targets"] = a.guide_targets
        if a.mixture_fraction is not None:
            WORKLOAD["mixture_fraction"] = a.mixture_fraction
    if a.warmup < 3:
        a.warmup = 3
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
