"""Renders a benchmark frame a few times, for profilers.

    python -m muon_gb300.profile_frame [--workload sphere_field] [--frames 1]
        [--warmup 2] [--mode exact|fast] [--width 512 --height 512 --spp 64]
        [--guided] [--train-steps 4]

With --guided the frames are guided renders (learned path guiding) and the
network trains for --train-steps Adam steps after each of them.

Used as the target of the ncu captures summarised in profiles/: the same
workload as bench.py, without its timing, e2e and CPU-baseline parts.
"""
from __future__ import annotations

import argparse

from . import Scene, native, scenes


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sphere_field", choices=sorted(scenes.WORKLOADS))
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--mode", default="exact", choices=["exact", "fast", "watertight"])
    ap.add_argument("--width", type=int, default=512)
    ap.add_argument("--height", type=int, default=512)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--guided", action="store_true")
    ap.add_argument("--train-steps", type=int, default=4)
    ap.add_argument("--batch", type=int, default=1 << 18)
    ap.add_argument("--mixture-fraction", type=float, default=0.0, help="guided ray mixture fraction (0: default)")
    ap.add_argument("--max-depth", type=int, default=None,
                    help="override the scene's max_depth (a depth-limited frame gives the queue lengths of its "
                         "first bounces: with next-event estimation, max depth d traces bounces 0..d-1)")
    a = ap.parse_args()
    text = scenes.WORKLOADS[a.workload](width=a.width, height=a.height, spp=a.spp)
    scene = Scene.from_string(text)
    mode = {"exact": native.ISECT_EXACT, "fast": native.ISECT_FAST, "watertight": native.ISECT_WATERTIGHT}[a.mode]
    over = {} if a.max_depth is None else {"max_depth": a.max_depth}
    if a.guided:
        import torch

        from . import Guide

        guide = Guide(scene, seed=1, batch=a.batch, mixture_fraction=a.mixture_fraction)
        n = scene.width * scene.height
        film = [torch.zeros((n, 3), dtype=torch.float64, device="cuda"),
                torch.zeros((n, 3), dtype=torch.float64, device="cuda"),
                torch.zeros(n, dtype=torch.int32, device="cuda")]
        for k in range(a.warmup + a.frames):
            guide.render_device(scene.params(intersect_mode=mode, seed=k), *[t.data_ptr() for t in film])
            guide.train(a.train_steps)
        torch.cuda.synchronize()
        print(f"guided {a.workload} {a.width}x{a.height}x{a.spp}: {guide.samples()} training samples")
        guide.close()
        scene.close()
        return
    for _ in range(a.warmup):
        scene.render(intersect_mode=mode, **over)
    for _ in range(a.frames):
        scene.render(intersect_mode=mode, **over)
    st = scene.stats()
    print(f"{a.workload} {a.width}x{a.height}x{a.spp}: {st['render_ms']:.3f} ms, "
          f"{st['kernel_launches']} launches, counted rays {st['primary_rays'] + st['secondary_rays']}")
    # units per kernel class in one frame, for scaling per-launch profiler
    # figures of this case to other sizes: extend traces (and shade / fold
    # process) extend_rays queue entries over extend_launches launches;
    # occlude traces occlude_rays over occlude_launches
    print("units " + " ".join(f"{k}={st[k]}" for k in ("extend_rays", "extend_launches", "occlude_rays",
                                                      "occlude_launches", "paths")))
    scene.close()


if __name__ == "__main__":
    main()
