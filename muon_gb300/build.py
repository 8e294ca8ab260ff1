"""Build the native parts in-tree: libmuon_gpu.so and the `muon` CLI.

CUDA sources compile with nvcc for sm_103a only; host C++ with g++. Objects go
to muon_gb300/lib/obj, outputs to muon_gb300/lib. Translation units compile in
parallel. Host code is compiled with -ffp-contract=off so float results do not
depend on whether the host CPU has fused multiply-add.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
CUDA_UNITS = ["kernels.cu", "noalloc.cu", "guide.cu", "bvh_build.cu", "bvh_sah.cu", "scene_records.cu"]
HOST_UNITS = ["scene_parser.cc", "mesh_io.cc", "scene_build.cc", "host_api.cc", "render.cc", "batch.cc",
              "guide_host.cc", "bvh_walk.cc"]
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"] + \
    os.environ.get("MUON_CXX_EXTRA", "").split()
NVFLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "--extended-lambda"] + os.environ.get("MUON_NVCC_EXTRA", "").split()


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose: bool = False) -> str:
    """Compiles everything that is out of date; returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "muon_gpu.h"))
    cuda_inc = os.path.join(CUDA_HOME, "include")
    jobs = []
    objs = []
    for unit in CUDA_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ, unit + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append([NVCC, *NVFLAGS, "-c", src, "-o", obj])
    for unit in HOST_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ, unit + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            jobs.append(["g++", *CXXFLAGS, "-I" + cuda_inc, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for _ in ex.map(_run, jobs):
            pass
    lib = os.path.join(LIB, "libmuon_gpu.so")
    if _newer(lib, objs):
        _run([NVCC, ARCH, "-shared", "-o", lib, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    cli_src = os.path.join(CSRC, "muon_cli.cc")
    cli = os.path.join(LIB, "muon")
    if _newer(cli, [cli_src, lib]):
        _run(["g++", *CXXFLAGS, cli_src, "-o", cli, "-L" + LIB, "-lmuon_gpu", "-Wl,-rpath,$ORIGIN"])
    return lib


def clean() -> None:
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    print(build())
