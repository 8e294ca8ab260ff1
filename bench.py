"""Benchmark of the GB300 path tracer: counted Mrays/s and guided vs plain
time to RMSE 1e-2, with the reference algorithm timed on the host cores.

Default run (one JSON line): the headline is the dense mesh, the largest
single-GPU configuration: a 1,310,720-triangle displaced icosphere (level 8,
GGX roughness 0.15) and 10,000 small clutter triangles in the Cornell box,
1024x1024, 256 spp, max depth 10, next-event estimation with MIS, BRDF
importance sampling, FP32 shading, FP64 film (muon_gb300.scenes.dense_mesh).
One step = one full frame. The same line carries the other configurations
as sub-objects, each measured the same way:
  cornell       Cornell box 256x256, 16 spp, depth 5, MIS, seed 1, plus the
                depth / normals / albedo integrators on the same scene
  sphere_field  512 seeded spheres, 512x512, 64 spp, depth 8
  batch64       64 seeded scenes of uneven size in one batched wavefront
  guiding       slit room 1024x1024: time to RMSE 1e-2, guided / plain

Metric: Mrays/s counted as the reference counts rays (primary + secondary,
the MIS-sampled ray included; shadow rays excluded, muon/integration.cc:34-38,
483), over device time with the scene resident and the film in device memory.
`e2e` is the same metric through the public API with host buffers: scene
creation (the description uploaded, records and BVH built on the device)
and the host film read-back inside every step.

Roofline of the dominant kernel class: algorithmic bytes per launch from the
host walk of the flattened BVH over sampled queue rays
(muon_gpu_probe_traversal; 32 B per box test, 64 B per primitive record,
plus the ray / hit records), over the kernel's CUDA-event time, against the
measured HBM copy peak; beside it the DRAM bytes the kernel moves (ncu, from
profiles/traffic.json) and the L1 / L2 read ceilings measured live.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload NAME] [--builder auto|gpu_sah|host|gpu]

`--workload NAME` measures one configuration alone. With N > 1 (torchrun),
every rank renders its own replica of each frame with a distinct seed (weak
scaling; the FP64 films of replicas merge by addition). `--impl reference`
times the reference algorithm (the oracle's restatement; the reference build
is x86-only) on all host cores, on a bounded sample of the same workload.
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
    # C0: the Cornell box of the reference's test scenes
    "cornell": {"workload": "cornell", "width": 256, "height": 256, "spp": 16, "max_depth": 5, "nee": "mis",
                "importance_sampling": "brdf", "russian_roulette": "off", "seed": 1},
    # C1: random sphere field
    "sphere_field": {"workload": "sphere_field", "spheres": 512, "width": 512, "height": 512, "spp": 64,
                     "max_depth": 8, "nee": "mis", "importance_sampling": "brdf", "seed": 1},
    # C2 (headline): 1,310,720-triangle displaced icosphere (level 8) + 10k clutter triangles in the Cornell box
    "dense_mesh": {"workload": "dense_mesh", "triangles": 1320756, "width": 1024, "height": 1024, "spp": 256,
                   "max_depth": 10, "nee": "mis", "importance_sampling": "brdf", "seed": 1},
    # C3: 64 seeded scenes of uneven size in one batched wavefront
    "batch64": {"workload": "batch64", "scenes": 64, "triangles": "log-uniform 1k-500k per scene",
                "resolutions": [128, 256, 512, 1024], "spp": "uniform 4-64", "max_depth": "uniform 4-10",
                "nee": "mis", "importance_sampling": "brdf", "seed": 1},
    # C4: learned path guiding, time to RMSE 1e-2 against a converged plain render, guided vs plain
    "guiding": {"workload": "slit_room", "triangles": 1310720 + 10000 + 14 + 2, "width": 1024, "height": 1024,
                "max_depth": 10, "nee": "mis", "importance_sampling": "brdf", "seed": 1, "target_rmse": 1e-2,
                "reference_spp": 8192, "pass_spp": 16, "train_steps_per_pass": 128, "train_passes": 2,
                "batch": 1 << 18, "guide_targets": "direct", "mixture_fraction": 0.95, "guided_bounces": 4},
}
HEADLINE = "dense_mesh"
SUB_WORKLOADS = ["sphere_field", "cornell", "batch64", "guiding"]
METRIC = "Mrays/s"
SLOTS = 2  # shadow slots per path vertex of the benchmark scenes: one area-light sample + the MIS ray
L2_NOTE = "flushed between steps (256 MiB write)"


def scene_text(w: dict) -> str:
    from muon_gb300 import scenes

    if w["workload"] == "dense_mesh":
        return scenes.dense_mesh(w["width"], w["height"], w["spp"], w["max_depth"], seed=w["seed"])
    if w["workload"] == "cornell":
        return scenes.cornell(w["width"], w["height"], w["spp"], w["max_depth"], w["seed"])
    return scenes.sphere_field(w["width"], w["height"], w["spp"], w["max_depth"], w["spheres"], w["seed"], w["nee"])


def dist_env() -> tuple[int, int, int]:
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


_INIT = [False]


def init_device():
    """Selects this rank's GPU, joins the process group (N > 1) and builds
    the native library in-tree."""
    import torch

    world, rank, local = dist_env()
    if not _INIT[0]:
        torch.cuda.set_device(local)
        if world > 1:
            torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
        from muon_gb300 import build as native_build

        native_build.build()
        _INIT[0] = True
    return world, rank, local


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


_CEIL: dict = {}


def ceilings() -> dict:
    """Read-bandwidth ceilings of this GPU measured now by the library's own
    kernel: L1 (32 KiB read by every block), L2 (24 MiB across the grid,
    bypassing L1), DRAM (4 GiB across the grid)."""
    if not _CEIL:
        import muon_gb300 as m

        _CEIL["l1_read_gbs"] = round(max(m.measure_read_bandwidth(0, 32 << 10, 500) for _ in range(3)), 1)
        _CEIL["l2_read_gbs"] = round(max(m.measure_read_bandwidth(1, 24 << 20, 400) for _ in range(3)), 1)
        _CEIL["dram_read_gbs"] = round(max(m.measure_read_bandwidth(2, 4 << 30, 2) for _ in range(3)), 1)
    return dict(_CEIL)


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


def algorithmic_bytes(probe: dict, st: dict, slots: int) -> dict:
    """Bytes each kernel class must move per frame by its algorithm, with the
    traversal work from the host walk of the flattened BVH (probe).

    Traversal (extend / occlude): 32 B per child box tested (a 64-B node holds
    two), 64 B per primitive record tested, plus the ray / hit records:
    extend reads a 32 B ray and writes an 8 B hit; occlude reads a 4 B queue
    entry, a 16 B origin and a 16 B direction.
    Shade, per shaded path: reads ray 32 + hit 8 + radiance 16 + throughput
    16, writes radiance 16 + slots 48*S (clear, value, direction); per
    continuation +48 (ray 32, throughput 16); per shadow ray +4 (queue entry).
    Fold, per shaded path: reads radiance 16 + slots 16*S + link 4, writes 16.
    """
    ext = 32 * probe["extend_box_tests"] + 64 * probe["extend_prim_tests"] + 40 * probe["extend_rays"]
    occ = 32 * probe["occlude_box_tests"] + 64 * probe["occlude_prim_tests"] + 36 * probe["occlude_rays"]
    shaded = st["extend_rays"]
    cont = max(0, st["extend_rays"] - st["primary_rays"])
    shade = shaded * (88 + 48 * slots) + 48 * cont + 4 * st["shadow_rays"]
    fold = shaded * (16 + 16 * slots + 4 + 16)
    return {"extend": ext, "occlude": occ, "shade": shade, "fold": fold}


def traffic(workload: str, kernel: str, rays_per_launch: float) -> dict | None:
    """DRAM bytes per launch of a traversal kernel: the bytes per ray of one
    ncu-captured launch of a smaller case (profiles/traffic.json, which gives
    the capture and its scaling) times this frame's rays per launch."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    entry = json.load(open(path)).get(workload, {}).get(kernel)
    if not entry:
        return None
    return {"bytes_per_launch": entry["bytes_per_ray"] * rays_per_launch,
            "source": f"profiles/traffic.json: {entry['bytes_per_ray']} DRAM bytes per ray (ncu, one launch of "
                      f"a 2^23-path wavefront) x {rays_per_launch:.0f} rays per launch"}


def cpu_baseline(text: str, w: dict, budget_s: float = 10.0, steps: int = 1) -> dict:
    """Counted Mrays/s of the reference algorithm (the oracle's restatement)
    on every host core, over its render time alone (the reference's Stats
    reports build and render time apart, muon/stats.cc:41-55): the scene is
    loaded once, then rendered at the spp that fills about budget_s."""
    from oracle import port

    threads = os.cpu_count() or 1
    ls = port.LoadedScene(text)
    try:
        c = ls.render(spp=1, seed=1, threads=threads)
        el1 = c["render_ns"] / 1e9
        spp = max(1, min(w["spp"], int(budget_s / max(el1, 1e-3))))
        rays, secs = 0, 0.0
        for k in range(steps):
            c = ls.render(spp=spp, seed=1 + k, threads=threads)
            rays += c["primary"] + c["secondary"]
            secs += c["render_ns"] / 1e9
    finally:
        ls.close()
    return {"value": round(rays / secs / 1e6, 3), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"full {w['width']}x{w['height']} frame at {spp} spp (of {w['spp']}) x {steps}, "
                      f"{secs:.1f} s of render on {threads} threads (scene loaded once)"}


def roofline(name: str, probe: dict, probe_stats: dict, last: dict) -> dict:
    """Roofline of the kernel class with the largest share of the frame."""
    alg = algorithmic_bytes(probe, probe_stats, SLOTS)
    times = {"extend": last["extend_ms"], "occlude": last["occlude_ms"], "shade": last["shade_ms"],
             "fold": last["fold_ms"]}
    dom = max(times, key=times.get)
    n_launch = {"extend": last["extend_launches"], "occlude": last["occlude_launches"],
                "shade": last["extend_launches"], "fold": last["extend_launches"]}[dom]
    per_launch_bytes = alg[dom] / max(1, n_launch)
    per_launch_ms = times[dom] / max(1, n_launch)
    pk = peaks()
    ce = ceilings()
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
    rays_per_launch = {"extend": probe_stats["extend_rays"] / max(1, probe_stats["extend_launches"]),
                       "occlude": probe_stats["occlude_rays"] / max(1, probe_stats["occlude_launches"])}
    tr = traffic(name, dom, rays_per_launch[dom]) if dom in rays_per_launch else None
    out = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
           "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": None, "peak_source": pk["source"],
           "per_launch_bytes": int(per_launch_bytes), "per_launch_ms": round(per_launch_ms, 4),
           "kernel_ms_per_step": {k: round(v, 3) for k, v in times.items()},
           "algorithmic_source": "host walk of the flattened BVH over sampled queue rays",
           "ceilings": ce, "frac_l2": round(achieved / ce["l2_read_gbs"], 4),
           "frac_l1": round(achieved / ce["l1_read_gbs"], 4)}
    if tr:
        out["traffic"] = int(tr["bytes_per_launch"])
        dram_gbs = tr["bytes_per_launch"] / (per_launch_ms * 1e-3) / 1e9
        out["frac_hbm_dram"] = round(dram_gbs / pk["hbm_gbs"], 4)
        out["traffic_source"] = tr["source"]
    # the host walk against the traversal kernels' own counters of the same render
    out["walk_vs_gpu_counters"] = {
        "extend_box_tests": round(probe["extend_box_tests"] / max(1, probe_stats["extend_box_tests"]), 4),
        "extend_prim_tests": round(probe["extend_prim_tests"] / max(1, probe_stats["extend_prim_tests"]), 4),
        "occlude_box_tests": round(probe["occlude_box_tests"] / max(1, probe_stats["occlude_box_tests"]), 4),
        "rays_walked": int(probe["extend_walked"]["rays"] + probe["occlude_walked"]["rays"])}
    return out


def desc_upload_bytes(parsed) -> int:
    """Bytes of a scene description that scene creation copies to the device
    (the description's arrays, as their C structs; the device computes the
    triangles' records from them)."""
    import ctypes as C

    from muon_gb300 import native

    d = parsed.desc
    return (d.num_triangles * C.sizeof(native.TriangleDesc) + d.num_spheres * C.sizeof(native.SphereDesc) +
            d.num_materials * C.sizeof(native.MaterialDesc) + d.num_lights * C.sizeof(native.LightDesc) +
            d.num_transforms * C.sizeof(native.TransformDesc))


def measure_frames(name: str, w: dict, steps: int, warmup: int, builder: str, with_cpu: bool) -> dict:
    """One step = one full frame of a single-scene workload (device time,
    film in device memory), then the same metric end to end through the
    public API, the roofline of the dominant kernel class and the CPU
    baseline. Returns the fields of a bench line."""
    import numpy as np
    import torch

    world, rank, local = init_device()
    import muon_gb300 as m
    from muon_gb300 import native, replicas

    text = scene_text(w)
    scene = m.Scene.from_string(text, builder=builder)
    seed = 1000 + rank
    # The timed frames render as a user's would (two wavefronts in flight);
    # the per-kernel split of the roofline comes from frames with every
    # kernel timed by CUDA events, which run the wavefronts one at a time.
    params = scene.params(seed=seed, intersect_mode=native.ISECT_EXACT)
    params_timed = scene.params(seed=seed, intersect_mode=native.ISECT_EXACT, flags=native.RENDER_TIMING)
    h, wd = scene.height, scene.width
    d_sum = torch.zeros((h, wd, 3), dtype=torch.float64, device="cuda")
    d_sq = torch.zeros((h, wd, 3), dtype=torch.float64, device="cuda")
    d_cnt = torch.zeros((h, wd), dtype=torch.int32, device="cuda")
    render = lambda p: scene.render_device(p, d_sum.data_ptr(), d_sq.data_ptr(), d_cnt.data_ptr())

    # traversal work of a frame, outside the timed region: host walk of
    # sampled queue rays, and the kernels' own counters of the same render
    probe = scene.probe_traversal(scene.params(seed=seed, intersect_mode=native.ISECT_EXACT), rays_per_queue=4096)
    probe_stats = scene.stats()

    stream = torch.cuda.ExternalStream(scene.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # 256 MiB > 129 MB L2
    for _ in range(warmup):
        render(params)
    torch.cuda.synchronize()

    st_steps = []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for k in range(steps):
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
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    counted = sum(s["primary_rays"] + s["secondary_rays"] for s in st_steps)
    launches = sum(s["kernel_launches"] for s in st_steps)
    dev_ms_max, counted_all = replicas.reduce_step(dev_ms, counted, device="cuda")
    value = counted_all / (dev_ms_max * 1e3)
    # per-kernel times (outside the timed region): the last of two timed frames
    for _ in range(2):
        flush.zero_()
        render(params_timed)
    kernel_stats = scene.stats()

    # end to end through the public API with host buffers
    e2e_steps = max(2, min(steps, 5))
    parsed = m.parse_string(text)
    desc_bytes = desc_upload_bytes(parsed)
    film_bytes = h * wd * (3 * 8 * 2 + 4)
    # the step's film comes back into pinned host memory, reused across steps
    host_film = m.FilmResult(torch.zeros((h, wd, 3), dtype=torch.float64).pin_memory().numpy(),
                             torch.zeros((h, wd, 3), dtype=torch.float64).pin_memory().numpy(),
                             torch.zeros((h, wd), dtype=torch.int32).pin_memory().numpy().view(np.uint32))
    m.Scene(parsed, builder=builder).render(params, out=host_film)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_counted = 0
    for _ in range(e2e_steps):
        sc = m.Scene(parsed, builder=builder)
        sc.render(params, out=host_film)
        s = sc.stats()
        e2e_counted += s["primary_rays"] + s["secondary_rays"]
        sc.close()
    e2e_value = e2e_counted / (time.perf_counter() - t0) / 1e6
    out = {
        "value": round(value, 2), "unit": METRIC, "ms_per_step": round(dev_ms_max / steps, 4), "steps": steps,
        "warmup": warmup, "counted_rays_per_step": counted // steps,
        "e2e": {"value": round(e2e_value, 2), "unit": METRIC, "h2d_bytes_per_step": int(desc_bytes),
                "d2h_bytes_per_step": int(film_bytes),
                "note": "scene create (description upload; records and BVH built on the device) + render + film "
                        "read-back into pinned host memory per step"},
        "gpu_launches": int(launches), "clocks": clocks.summary(), "wall_s": round(wall, 3),
    }
    if rank == 0:
        out["roofline"] = roofline(name, probe, probe_stats, kernel_stats)
        if with_cpu and world == 1:
            out["cpu_baseline"] = cpu_baseline(text, w)
    scene.close()
    return out


def measure_deterministic(w: dict, steps: int, warmup: int) -> dict:
    """The depth, normals and albedo integrators (muon/integration.cc:47-72)
    on the C0 scene at 1 spp: one closest hit per pixel, device time."""
    import torch

    init_device()
    import muon_gb300 as m
    from muon_gb300 import native

    scene = m.Scene.from_string(scene_text(w))
    h, wd = scene.height, scene.width
    film = [torch.zeros((h, wd, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, wd, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, wd), dtype=torch.int32, device="cuda")]
    stream = torch.cuda.ExternalStream(scene.stream())
    out = {}
    for integ in ("depth", "normals", "albedo"):
        p = scene.params(integrator=integ, pixel_samples=1, intersect_mode=native.ISECT_EXACT)
        for _ in range(warmup):
            scene.render_device(p, *[x.data_ptr() for x in film])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream.wait_stream(torch.cuda.current_stream())
        e0.record(stream)
        for _ in range(steps):
            scene.render_device(p, *[x.data_ptr() for x in film])
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        rays = scene.stats()["primary_rays"]
        out[integ] = {"ms_per_frame": round(ms, 4), "value": round(rays / (ms * 1e3), 1), "unit": METRIC}
    scene.close()
    return out


def batch_texts(w: dict) -> list[str]:
    from muon_gb300 import scenes

    return [scenes.batch_scene(i, w["seed"]) for i in range(w["scenes"])]


def measure_batch(w: dict, steps: int, warmup: int, builder: str, with_cpu: bool) -> dict:
    """One step = one batched render of all 64 scenes
    (muon_gpu_batch_render_device)."""
    import torch

    world, rank, local = init_device()
    import muon_gb300 as m
    from muon_gb300 import native, replicas

    texts = batch_texts(w)
    parsed = [m.parse_string(t) for t in texts]
    sc = [m.Scene(p, builder=builder) for p in parsed]
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
    for _ in range(warmup):
        render()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    times, counted, lat, launches = [], 0, [], 0
    with ClockSampler(local) as clocks:
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            render()
            total, per = batch.stats()
            times.append(total["render_ms"])
            counted += total["primary_rays"] + total["secondary_rays"]
            lat += [p["done_ms"] for p in per]
            launches += total["kernel_launches"]
    dev_ms, counted = replicas.reduce_step(sum(times), counted, device="cuda")
    value = counted / (dev_ms * 1e3)
    # the same scenes rendered one at a time (each its own graph, device
    # time): what batching them into one wavefront buys, and what it costs a
    # scene in latency
    alone = []
    for s_, p_, f_ in zip(sc, params, films):
        s_.render_device(p_, *[x.data_ptr() for x in f_])  # first render of a configuration: no graph yet
        s_.render_device(p_, *[x.data_ptr() for x in f_])
        s_.render_device(p_, *[x.data_ptr() for x in f_])
        alone.append(s_.stats()["render_ms"])
    torch.cuda.synchronize()
    # end to end: scene uploads (BVH builds), batch merge, render, host films back
    e2e_steps = 2
    h2d = sum(desc_upload_bytes(p) for p in parsed)
    d2h = sum(s.width * s.height * (3 * 8 * 2 + 4) for s in sc)
    t0 = time.perf_counter()
    e2e_counted = 0
    for _ in range(e2e_steps):
        scs = [m.Scene(p, builder=builder) for p in parsed]
        b2 = m.Batch(scs)
        b2.render(params)
        tot, _ = b2.stats()
        e2e_counted += tot["primary_rays"] + tot["secondary_rays"]
        b2.close()
        for s in scs:
            s.close()
    e2e_value = e2e_counted / (time.perf_counter() - t0) / 1e6
    lat_sorted = sorted(lat)
    pct = lambda q: lat_sorted[min(len(lat_sorted) - 1, int(q * len(lat_sorted)))]
    out = {
        "value": round(value, 2), "unit": METRIC, "ms_per_step": round(dev_ms / steps, 3), "steps": steps,
        "warmup": warmup, "total_triangles": int(sum(p.desc.num_triangles for p in parsed)),
        "paths_per_step": int(total["paths"]),
        "latency_ms": {"p50": round(pct(0.50), 3), "p99": round(pct(0.99), 3), "max": round(lat_sorted[-1], 3),
                       "note": "per scene: batch start to its film complete"},
        "alone_ms": {"sum": round(sum(alone), 1), "p50": round(sorted(alone)[len(alone) // 2], 3),
                     "p99": round(sorted(alone)[min(len(alone) - 1, int(0.99 * len(alone)))], 3),
                     "max": round(max(alone), 3),
                     "note": "each scene rendered by itself (its own CUDA graph), device time"},
        "autotune": dict(tune, seconds=round(t_tune, 2)),
        "e2e": {"value": round(e2e_value, 2), "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "note": "64 scene uploads (BVH builds) + batch merge + render + host films back per step"},
        "gpu_launches": int(launches), "clocks": clocks.summary(),
    }
    if with_cpu and world == 1 and rank == 0:
        from oracle import port

        threads = os.cpu_count() or 1
        rays, secs = 0, 0.0
        for i in range(4):
            ls = port.LoadedScene(texts[i])
            c = ls.render(spp=1, seed=1, threads=threads)
            ls.close()
            rays += c["primary"] + c["secondary"]
            secs += c["render_ns"] / 1e9
        out["cpu_baseline"] = {"value": round(rays / secs / 1e6, 3), "unit": METRIC, "cores": threads,
                               "kind": "port", "sample": f"scenes 0-3 of the batch at 1 spp, {secs:.1f} s of render "
                                                         f"on {threads} threads"}
    batch.close()
    for s in sc:
        s.close()
    return out


def measure_guiding(w: dict) -> dict:
    """Time to reach RMSE 1e-2 against a converged plain render of the slit
    room: the plain GPU tracer and the guided one (training time included),
    both rendering progressive passes of `pass_spp` samples; device time with
    CUDA events, the RMSE evaluations between passes excluded."""
    import torch

    init_device()
    import muon_gb300 as m
    from muon_gb300 import native, scenes

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
    del ref

    def rmse(f):
        img = f[0] / f[2].clamp(min=1)[..., None].double()
        return float(torch.sqrt(((img - ref_img) ** 2).mean()))

    def progressive(render_pass, train=None, max_passes=4096):
        f = film()
        dev_ms, spp, passes, counted, launches = 0.0, 0, 0, 0, 0
        trace = []
        while passes < max_passes:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream.wait_stream(torch.cuda.current_stream())
            e0.record(stream)
            c, l = render_pass(f, spp)
            counted += c
            launches += l
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
        return dev_ms, spp, err, counted, launches, trace

    # passes launch kernel by kernel: a graph would be captured again for
    # every pass (its sample offset changes)
    def plain_pass(f, spp):
        scene.render_device(scene.params(pixel_samples=w["pass_spp"], seed=11, sample_offset=spp,
                                         flags=native.RENDER_NO_GRAPH | (native.RENDER_ACCUMULATE if spp else 0)),
                            *ptr(f))
        st = scene.stats()
        return st["primary_rays"] + st["secondary_rays"], st["kernel_launches"]

    guide = m.Guide(scene, seed=w["seed"], batch=w["batch"], mixture_fraction=w["mixture_fraction"],
                    record_bounces=w["guided_bounces"],
                    targets=native.GUIDE_DIRECT if w["guide_targets"] == "direct" else native.GUIDE_ALL)

    def guided_pass(f, spp):
        guide.render_device(scene.params(pixel_samples=w["pass_spp"], seed=12, sample_offset=spp,
                                         flags=native.RENDER_NO_GRAPH | (native.RENDER_ACCUMULATE if spp else 0)),
                            *ptr(f))
        st = scene.stats()
        return st["primary_rays"] + st["secondary_rays"], st["kernel_launches"]

    passes_trained = [0]

    def train():
        # online training during the first passes, then the network is frozen
        if passes_trained[0] < w["train_passes"]:
            guide.train(w["train_steps_per_pass"])
            passes_trained[0] += 1

    plain_ms, plain_spp, plain_err, plain_rays, plain_l, plain_trace = progressive(plain_pass)
    guided_ms, guided_spp, guided_err, guided_rays, guided_l, guided_trace = progressive(guided_pass, train=train)
    samples = guide.samples()
    guide.close()
    scene.close()
    return {
        "value": round(guided_ms / plain_ms, 4), "unit": "ratio", "metric": "time-to-RMSE 1e-2 (guided / plain)",
        "higher_is_better": False, "reference_seconds": round(ref_s, 2),
        "plain": {"ms": round(plain_ms, 1), "spp": plain_spp, "rmse": round(plain_err, 5),
                  "mrays_per_s": round(plain_rays / (plain_ms * 1e3), 1)},
        "guided": {"ms": round(guided_ms, 1), "spp": guided_spp, "rmse": round(guided_err, 5),
                   "mrays_per_s": round(guided_rays / (guided_ms * 1e3), 1), "samples": samples},
        "gpu_launches": int(plain_l + guided_l),
        "trace_plain": plain_trace[-4:], "trace_guided": guided_trace[-4:],
    }


def run_reference(args, name: str) -> None:
    """The reference algorithm (the oracle's restatement of it) on all host
    cores: each step renders a bounded sample of the workload (whole frames
    at a reduced spp; for the batch, its first scene at 1 spp), the scene
    loaded once; counted Mrays/s over render time."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as oracle_build
    from oracle import port

    oracle_build.build()
    threads = os.cpu_count() or 1
    w = WORKLOADS[name]
    if name == "batch64":
        text, spp = batch_texts(w)[0], 1
        sample = "scene 0 of the batch at 1 spp per step"
    elif name == "guiding":
        from muon_gb300 import scenes

        text = scenes.slit_room(w["width"], w["height"], 16, w["max_depth"], seed=w["seed"])
        spp = 1
        sample = "full 1024x1024 slit-room frame at 1 spp per step (plain path tracer)"
    else:
        text = scene_text(w)
        spp = None
    ls = port.LoadedScene(text)
    if spp is None:
        c = ls.render(spp=1, seed=1, threads=threads)
        spp = max(1, min(w["spp"], int(4.0 / max(c["render_ns"] / 1e9, 1e-3))))
        sample = f"full {w['width']}x{w['height']} frame at {spp} spp (of {w['spp']}) per step, scene loaded once"
    for k in range(args.warmup):
        ls.render(spp=1, seed=100 + k, threads=threads)
    rays, secs = [], []
    for k in range(args.steps):
        c = ls.render(spp=spp, seed=1 + k, threads=threads)
        rays.append(c["primary"] + c["secondary"])
        secs.append(c["render_ns"] / 1e9)
    ls.close()
    value = sum(rays) / sum(secs) / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(secs) / len(secs), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic (seeded {w['workload'].replace('_', ' ')})",
            "config": dict(w, parallelism=f"host threads {threads}"),
            "cpu_baseline": {"value": round(value, 3), "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def base_line(name: str, res: dict, world: int, builder: str) -> dict:
    w = WORKLOADS[name]
    line = {"metric": METRIC, "value": res["value"], "unit": METRIC, "n_gpus": world, "steps": res["steps"],
            "warmup": res["warmup"], "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": f"synthetic (seeded {w['workload'].replace('_', ' ')})",
            "config": dict(w, parallelism=f"replicas{world}", intersect_mode="exact", bvh_builder=builder,
                           l2=L2_NOTE)}
    if "counted_rays_per_step" in res:
        line["config"]["counted_rays_per_step"] = res["counted_rays_per_step"]
    for k in ("e2e", "gpu_launches", "roofline", "clocks", "wall_s", "cpu_baseline", "latency_ms", "autotune"):
        if k in res:
            line[k] = res[k]
    return line


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["all"] + sorted(WORKLOADS), default="all",
                    help="all (default): the dense mesh as the headline with the other configurations as "
                         "sub-objects of the same line; or one configuration alone")
    ap.add_argument("--builder", choices=["auto", "gpu_sah", "host", "gpu"], default="auto",
                    help="BVH builder: binned SAH on the GPU (the same tree as the host's; 'auto', the default, "
                         "builds scenes of fewer than 256 primitives on the host), binned SAH on the host threads, "
                         "or the linear BVH built on the GPU")
    ap.add_argument("--guide-targets", choices=["direct", "all"], default=None,
                    help="guiding workload: what the network learns (default: direct light)")
    ap.add_argument("--mixture-fraction", type=float, default=None,
                    help="guiding workload: probability that a guided ray samples the mixture")
    ap.add_argument("--no-subs", action="store_true", help="default run: the headline only")
    a = ap.parse_args()
    if a.guide_targets:
        WORKLOADS["guiding"]["guide_targets"] = a.guide_targets
    if a.mixture_fraction is not None:
        WORKLOADS["guiding"]["mixture_fraction"] = a.mixture_fraction
    a.warmup = max(a.warmup, 3)
    name = HEADLINE if a.workload == "all" else a.workload
    if a.impl == "reference":
        return run_reference(a, name)
    world, rank, _ = init_device()
    if name == "guiding":
        res = measure_guiding(WORKLOADS["guiding"])
        if rank == 0:
            line = {"metric": res.pop("metric"), "value": res.pop("value"), "unit": "ratio", "n_gpus": 1,
                    "steps": 1, "warmup": 0, "higher_is_better": False, "scaling": "none", "vs_baseline": None,
                    "dtype": "f32 (bf16 network)", "data": "synthetic (seeded slit room)",
                    "config": dict(WORKLOADS["guiding"])}
            line.update(res)
            print(json.dumps(line), flush=True)
        return
    if name == "batch64":
        res = measure_batch(WORKLOADS[name], a.steps, a.warmup, a.builder, with_cpu=True)
    else:
        res = measure_frames(name, WORKLOADS[name], a.steps, a.warmup, a.builder, with_cpu=True)
    line = base_line(name, res, world, a.builder)
    if name == "cornell":
        line["deterministic"] = measure_deterministic(WORKLOADS["cornell"], a.steps, a.warmup)
    if a.workload == "all" and not a.no_subs and world == 1:
        # the other configurations, measured the same way on this GPU
        sub_steps = {"sphere_field": a.steps, "cornell": a.steps, "batch64": min(a.steps, 3)}
        for sub in SUB_WORKLOADS:
            t0 = time.perf_counter()
            if sub == "guiding":
                r = measure_guiding(WORKLOADS["guiding"])
                r["config"] = dict(WORKLOADS["guiding"])
            elif sub == "batch64":
                r = measure_batch(WORKLOADS[sub], sub_steps[sub], a.warmup, a.builder, with_cpu=True)
                r["config"] = dict(WORKLOADS[sub])
            else:
                r = measure_frames(sub, WORKLOADS[sub], sub_steps[sub], a.warmup, a.builder, with_cpu=True)
                r["config"] = dict(WORKLOADS[sub])
                if sub == "cornell":
                    r["deterministic"] = measure_deterministic(WORKLOADS["cornell"], a.steps, a.warmup)
            r["seconds"] = round(time.perf_counter() - t0, 1)
            line[sub] = r
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
