"""Times the reference build (oracle/_ref/muon_ref, the reference's own CLI and
Renderer) and the oracle's restatement (oracle/port.py) on the same scenes,
host threads and samples per pixel, so that the port's CPU baseline on a
machine where the reference build cannot run (the aarch64 GPU host) can be
read as the reference's. Test infrastructure: it needs the reference build,
which exists only where the reference sources are (oracle/Makefile).

Both report counted Mrays/s (primary + secondary rays, muon/stats.h:11-44)
over render time alone (the reference prints build and render time apart,
muon/stats.cc:41-55; the port times them apart too).

  python oracle/compare_speed.py [--threads N] [--repeats R]
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

REF = os.path.join(HERE, "_ref", "muon_ref")

# (name, generator call, spp): the benchmark scenes at a reduced spp
CASES = [
    ("cornell 256x256", "scenes.cornell(256, 256, 16, 5, 1)", 16),
    ("sphere field 512x512", "scenes.sphere_field(512, 512, 64, 8)", 4),
    ("dense mesh 1024x1024", "scenes.dense_mesh(1024, 1024, 256, 10)", 1),
]


def reference(text: str, spp: int, threads: int) -> tuple[float, float, int]:
    """(Mrays/s, render seconds, counted rays) of the reference CLI."""
    text = re.sub(r"pixel_samples \d+", f"pixel_samples {spp}", text)
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "s.muon")
        open(sp, "w").write(text)
        r = subprocess.run([REF, f"--scene={sp}", f"--output={os.path.join(td, 'o.ppm')}",
                            f"--parallelism={threads}"], capture_output=True, text=True, check=True)
    out = r.stdout + r.stderr
    secs = float(re.search(r"Render time\s*:\s*([\d.]+)", out).group(1))
    rays = int(re.search(r"Primary rays\s*:\s*(\d+)", out).group(1)) + \
        int(re.search(r"Secondary rays\s*:\s*(\d+)", out).group(1))
    return rays / secs / 1e6, secs, rays


def port(text: str, spp: int, threads: int) -> tuple[float, float, int]:
    from oracle import port as P

    ls = P.LoadedScene(text)
    c = ls.render(spp=spp, threads=threads)
    ls.close()
    secs = c["render_ns"] / 1e9
    rays = c["primary"] + c["secondary"]
    return rays / secs / 1e6, secs, rays


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--repeats", type=int, default=2)
    a = ap.parse_args()
    from muon_gb300 import scenes  # noqa: F401  (used by the generator calls)

    print(f"threads {a.threads}; counted Mrays/s over render time, best of {a.repeats}")
    print(f"{'scene':24s} {'spp':>4s} {'reference':>10s} {'port':>10s} {'port/ref':>9s}")
    for name, call, spp in CASES:
        text = eval(call)
        ref = max(reference(text, spp, a.threads)[0] for _ in range(a.repeats))
        prt = max(port(text, spp, a.threads)[0] for _ in range(a.repeats))
        print(f"{name:24s} {spp:4d} {ref:10.3f} {prt:10.3f} {prt / ref:9.3f}", flush=True)


if __name__ == "__main__":
    main()
