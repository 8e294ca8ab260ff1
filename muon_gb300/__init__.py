"""GB300 rendering path of the muon path tracer.

Python mirror of the reference renderer's interface for its hot path
(muon/renderer.cc Renderer::Render, muon/parser.cc Parser::Parse,
muon/acceleration.h Structure::Intersect/HasIntersection, muon/film.cc
Film::WriteOutput) over the C ABI in include/muon_gpu.h.

    scene = muon_gb300.Scene.from_file("cornell.muon")
    film = scene.render()                 # settings from the scene file
    film.write("out.png", scene.gamma)

Rendering runs on the GPU only; a missing native library or CUDA device is an
error, never a silent CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native
from .native import MuonError, check, load

__all__ = ["Scene", "FilmResult", "MuonError", "render_file", "parse_file", "parse_string"]


class ParsedScene:
    """A parsed .muon scene (host memory), Parser::Parse's SceneConfig."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        self.desc = native.SceneDesc()
        self.params = native.RenderParams()
        check(load().muon_parsed_scene_desc(self._h, C.byref(self.desc), C.byref(self.params)))

    @property
    def gamma(self) -> float:
        return float(load().muon_parsed_scene_gamma(self._h))

    @property
    def output(self) -> str | None:
        o = load().muon_parsed_scene_output(self._h)
        return o.decode() if o else None

    @property
    def warnings(self) -> int:
        return int(load().muon_parsed_scene_warnings(self._h))

    def close(self) -> None:
        if self._h:
            load().muon_parsed_scene_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def walk_rays(parsed: ParsedScene, origins: np.ndarray, directions: np.ndarray, tmax: np.ndarray | None = None,
              any_hit: bool = False, intersect_mode: int = native.ISECT_EXACT) -> tuple[np.ndarray, dict]:
    """Host walk of the scene's BVH (muon_walk_rays, no GPU): per ray the
    parse-order id of the primitive hit (-1: none), and the traversal counts."""
    n = len(origins)
    rays = np.zeros((n, 6), dtype=np.float32)
    rays[:, :3] = origins
    rays[:, 3:] = directions
    tm = None if tmax is None else np.ascontiguousarray(tmax, dtype=np.float32)
    ids = np.zeros(n, dtype=np.int32)
    cnt = native.WalkCounts()
    desc = parsed.desc
    # the BVH a Scene builds by default: binned SAH on the host
    desc.acceleration, desc.builder = native.ACCEL_BVH, 0
    desc.partition_strategy, desc.max_leaf_size = native.PARTITION["sah"], 0
    check(load().muon_walk_rays(C.byref(desc), rays.ctypes.data_as(C.POINTER(native.Ray)),
                                None if tm is None else tm.ctypes.data_as(C.POINTER(C.c_float)), n, int(any_hit),
                                intersect_mode, ids.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(cnt)))
    return ids, {k: getattr(cnt, k) for k, _ in native.WalkCounts._fields_}


def measure_read_bandwidth(level: int, nbytes: int, passes: int) -> float:
    """GB/s of a read-bandwidth ceiling on the current device: level 0 L1,
    1 L2, 2 DRAM (muon_gpu_measure_read_bandwidth)."""
    v = C.c_double()
    check(load().muon_gpu_measure_read_bandwidth(level, nbytes, passes, C.byref(v)))
    return v.value


def parse_file(path: str) -> ParsedScene:
    h = C.c_void_p()
    check(load().muon_parse_scene_file(path.encode(), C.byref(h)))
    return ParsedScene(h.value)


def parse_string(text: str, base_dir: str = ".") -> ParsedScene:
    h = C.c_void_p()
    check(load().muon_parse_scene_string(text.encode(), base_dir.encode(), C.byref(h)))
    return ParsedScene(h.value)


@dataclass
class FilmResult:
    """FP64 film: per-pixel sums, sums of squares and sample counts."""

    sum: np.ndarray     # (H, W, 3) float64
    sum_sq: np.ndarray  # (H, W, 3) float64
    count: np.ndarray   # (H, W) uint32

    @property
    def width(self) -> int:
        return self.sum.shape[1]

    @property
    def height(self) -> int:
        return self.sum.shape[0]

    def mean(self) -> np.ndarray:
        n = np.maximum(self.count, 1)[..., None].astype(np.float64)
        return self.sum / n

    def variance_of_mean(self) -> np.ndarray:
        n = np.maximum(self.count, 1)[..., None].astype(np.float64)
        m = self.sum / n
        var = np.maximum(self.sum_sq / n - m * m, 0.0) * n / np.maximum(n - 1, 1)
        return var / n

    def _cfilm(self):
        f = native.Film()
        f.width, f.height = self.width, self.height
        f.sum = self.sum.ctypes.data_as(C.POINTER(C.c_double))
        f.sum_sq = self.sum_sq.ctypes.data_as(C.POINTER(C.c_double))
        f.count = self.count.ctypes.data_as(C.POINTER(C.c_uint32))
        return f

    def tonemap(self, gamma: float = 1.0) -> np.ndarray:
        """8-bit RGB exactly as Film::WriteOutput forms it (muon/film.cc:21-43)."""
        out = np.zeros((self.height, self.width, 3), dtype=np.uint8)
        f = self._cfilm()
        check(load().muon_film_tonemap(C.byref(f), C.c_float(gamma), out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out

    def write(self, path: str, gamma: float = 1.0) -> None:
        f = self._cfilm()
        check(load().muon_film_write(C.byref(f), C.c_float(gamma), path.encode()))


# Below this many primitives the host builds the SAH tree faster than the
# device's launches and synchronisations (measured on a GB300: 36 primitives
# 0.20 ms on the host vs 0.39 ms on the device; 516 primitives 1.04 vs 0.55 ms).
DEVICE_BUILD_MIN_PRIMS = 256


class Scene:
    """A scene resident on the GPU (Structure::Init + upload).

    builder: "gpu_sah" the binned-SAH BVH built on the device, the same tree
    as "host" (the same builder on the host threads); "auto" (default) the
    device build from DEVICE_BUILD_MIN_PRIMS primitives up, else the host
    build; "gpu" the linear BVH (faster to build, slower to traverse). Other
    partition strategies than SAH build on the host."""

    def __init__(self, parsed: ParsedScene, acceleration: str = "bvh", partition_strategy: str = "sah",
                 max_leaf_size: int = 0, builder: str = "auto"):
        self.parsed = parsed
        desc = parsed.desc
        desc.acceleration = native.ACCEL_LINEAR if acceleration == "linear" else native.ACCEL_BVH
        desc.partition_strategy = native.PARTITION[partition_strategy]
        if builder == "auto":
            builder = "gpu_sah" if desc.num_triangles + desc.num_spheres >= DEVICE_BUILD_MIN_PRIMS else "host"
        if partition_strategy != "sah" and builder == "gpu_sah":
            builder = "host"
        desc.max_leaf_size = max_leaf_size
        if builder not in native.BUILDER:
            raise ValueError(f"unknown BVH builder {builder!r}")
        desc.builder = native.BUILDER[builder]
        h = C.c_void_p()
        check(load().muon_gpu_scene_create(C.byref(desc), C.byref(h)))
        self._h = h
        self.width, self.height = desc.width, desc.height

    @classmethod
    def from_file(cls, path: str, **kw) -> "Scene":
        return cls(parse_file(path), **kw)

    @classmethod
    def from_string(cls, text: str, **kw) -> "Scene":
        return cls(parse_string(text), **kw)

    @property
    def gamma(self) -> float:
        return self.parsed.gamma

    def params(self, **overrides) -> native.RenderParams:
        """The scene file's render settings with keyword overrides applied."""
        p = native.RenderParams()
        C.pointer(p)[0] = self.parsed.params
        for k, v in overrides.items():
            if k == "integrator" and isinstance(v, str):
                v = native.INTEGRATORS[v]
            elif k == "next_event_estimation" and isinstance(v, str):
                v = native.NEE[v]
            elif k == "importance_sampling" and isinstance(v, str):
                v = native.IMPORTANCE[v]
            elif k == "intersect_mode" and isinstance(v, str):
                v = {"fast": native.ISECT_FAST, "watertight": native.ISECT_WATERTIGHT, "exact": native.ISECT_EXACT}[v]
            setattr(p, k, v)
        return p

    def render(self, params: native.RenderParams | None = None, out: FilmResult | None = None,
               **overrides) -> FilmResult:
        """Renders the whole film (Renderer::Render's sample loop) on the GPU.
        `out`, if given, receives the film (C-contiguous arrays of the film's
        shape; pinned host memory makes the copies fastest)."""
        p = params if params is not None else self.params(**overrides)
        h, w = self.height, self.width
        if out is not None:
            film = out
            ok = (film.sum.shape == (h, w, 3) and film.sum_sq.shape == (h, w, 3) and film.count.shape == (h, w)
                  and film.sum.dtype == np.float64 and film.sum_sq.dtype == np.float64
                  and film.count.dtype == np.uint32
                  and all(a.flags["C_CONTIGUOUS"] for a in (film.sum, film.sum_sq, film.count)))
            if not ok:
                raise ValueError("out film does not match the scene's film")
        else:
            film = FilmResult(np.zeros((h, w, 3)), np.zeros((h, w, 3)), np.zeros((h, w), dtype=np.uint32))
        f = film._cfilm()
        check(load().muon_gpu_render(self._h, C.byref(p), C.byref(f)))
        return film

    def render_device(self, params: native.RenderParams, d_sum: int, d_sum_sq: int, d_count: int) -> None:
        """Renders into a film already in device memory (raw device pointers)."""
        check(load().muon_gpu_render_device(self._h, C.byref(params), C.c_void_p(d_sum), C.c_void_p(d_sum_sq),
                                             C.c_void_p(d_count)))

    def intersect(self, origins: np.ndarray, directions: np.ndarray, intersect_mode: int = native.ISECT_EXACT):
        """Closest hits (Structure::Intersect) for a batch of rays.

        Returns (distance, prim_id, position, normal); prim_id is the primitive's
        index in scene-file order, -1 on a miss.
        """
        n = len(origins)
        rays = np.zeros((n, 6), dtype=np.float32)
        rays[:, :3] = origins
        rays[:, 3:] = directions
        hits = np.zeros((n, 8), dtype=np.float32)
        check(load().muon_gpu_intersect(self._h, rays.ctypes.data_as(C.POINTER(native.Ray)), n, intersect_mode,
                                        hits.ctypes.data_as(C.POINTER(native.Hit))))
        return hits[:, 0].copy(), hits[:, 1].view(np.int32).copy(), hits[:, 2:5].copy(), hits[:, 5:8].copy()

    def occluded(self, origins: np.ndarray, directions: np.ndarray, max_distance: np.ndarray,
                 intersect_mode: int = native.ISECT_EXACT) -> np.ndarray:
        """Any hit closer than max_distance (Structure::HasIntersection)."""
        n = len(origins)
        rays = np.zeros((n, 6), dtype=np.float32)
        rays[:, :3] = origins
        rays[:, 3:] = directions
        md = np.ascontiguousarray(max_distance, dtype=np.float32)
        out = np.zeros(n, dtype=np.uint8)
        check(load().muon_gpu_occluded(self._h, rays.ctypes.data_as(C.POINTER(native.Ray)),
                                       md.ctypes.data_as(C.POINTER(C.c_float)), n, intersect_mode,
                                       out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out.astype(bool)

    def probe_traversal(self, params: native.RenderParams, rays_per_queue: int = 4096) -> dict:
        """Traversal work of a render counted by the host walk of sampled
        queue rays (muon_gpu_probe_traversal); stats() then holds the GPU
        kernels' own counters of the same render."""
        pr = native.TraversalProbe()
        check(load().muon_gpu_probe_traversal(self._h, C.byref(params), rays_per_queue, C.byref(pr)))
        walked = lambda w: {k: getattr(w, k) for k, _ in native.WalkCounts._fields_}
        out = {k: getattr(pr, k) for k, _ in native.TraversalProbe._fields_ if not k.endswith("_walked")}
        out["extend_walked"] = walked(pr.extend_walked)
        out["occlude_walked"] = walked(pr.occlude_walked)
        return out

    def stats(self) -> dict:
        s = native.Stats()
        check(load().muon_gpu_stats(self._h, C.byref(s)))
        return {name: getattr(s, name) for name, _ in native.Stats._fields_}

    def stream(self) -> int:
        """The cudaStream_t this scene launches on, as an integer handle."""
        v = C.c_void_p()
        check(load().muon_gpu_scene_stream(self._h, C.byref(v)))
        return v.value or 0

    def bvh(self) -> tuple[dict, np.ndarray, np.ndarray, np.ndarray]:
        """The scene's BVH (muon_gpu_scene_bvh): build statistics, the nodes as
        an (n, 16) float32 array (columns 12 and 13 are the int32 links, read
        them through .view(np.int32)), and per record slot in leaf order the
        primitive id and the leaf-end flag."""
        info = native.BvhInfo()
        check(load().muon_gpu_scene_bvh(self._h, C.byref(info), None, None, None))
        nodes = np.zeros((info.nodes, 16), dtype=np.float32)
        prim = np.zeros(info.slots, dtype=np.int32)
        last = np.zeros(info.slots, dtype=np.uint8)
        check(load().muon_gpu_scene_bvh(self._h, C.byref(info), nodes.ctypes.data_as(C.c_void_p),
                                        prim.ctypes.data_as(C.POINTER(C.c_int32)),
                                        last.ctypes.data_as(C.POINTER(C.c_uint8))))
        return {k: getattr(info, k) for k, _ in native.BvhInfo._fields_}, nodes, prim, last

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().muon_gpu_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several GPU scenes rendered by one wavefront (muon_gpu_batch_*)."""

    def __init__(self, scenes: list[Scene]):
        self.scenes = list(scenes)
        hs = (C.c_void_p * len(self.scenes))(*[s._h for s in self.scenes])
        h = C.c_void_p()
        check(load().muon_gpu_batch_create(hs, len(self.scenes), C.byref(h)))
        self._h = h

    def _params(self, params):
        arr = (native.RenderParams * len(self.scenes))()
        for i, p in enumerate(params):
            arr[i] = p
        return arr

    def render(self, params: list[native.RenderParams]) -> list[FilmResult]:
        films = [FilmResult(np.zeros((s.height, s.width, 3)), np.zeros((s.height, s.width, 3)),
                            np.zeros((s.height, s.width), dtype=np.uint32)) for s in self.scenes]
        cf = (native.Film * len(films))(*[f._cfilm() for f in films])
        check(load().muon_gpu_batch_render(self._h, self._params(params), cf))
        return films

    def render_device(self, params: list[native.RenderParams], d_sum: list[int], d_sum_sq: list[int],
                      d_count: list[int]) -> None:
        n = len(self.scenes)
        arr = lambda xs: (C.c_void_p * n)(*[C.c_void_p(x) for x in xs])
        check(load().muon_gpu_batch_render_device(self._h, self._params(params), arr(d_sum), arr(d_sum_sq),
                                                  arr(d_count)))

    def autotune(self, params: list[native.RenderParams]) -> dict:
        t = native.BatchTuning()
        check(load().muon_gpu_batch_autotune(self._h, self._params(params), C.byref(t)))
        return {name: getattr(t, name) for name, _ in native.BatchTuning._fields_ if name != "pad"}

    def stats(self) -> tuple[dict, list[dict]]:
        s = native.Stats()
        per = (native.BatchSceneStats * len(self.scenes))()
        check(load().muon_gpu_batch_stats(self._h, C.byref(s), per))
        total = {name: getattr(s, name) for name, _ in native.Stats._fields_}
        return total, [{"primary_rays": x.primary_rays, "done_ms": x.done_ms} for x in per]

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().muon_gpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Guide:
    """Learned path guiding for one scene (muon_gpu_guide_*)."""

    def __init__(self, scene: Scene, **config):
        self.scene = scene
        cfg = native.GuideConfig()
        for k, v in config.items():
            setattr(cfg, k, v)
        h = C.c_void_p()
        check(load().muon_gpu_guide_create(scene._h, C.byref(cfg), C.byref(h)))
        self._h = h

    def render_device(self, params: native.RenderParams, d_sum: int, d_sum_sq: int, d_count: int) -> None:
        check(load().muon_gpu_guide_render_device(self._h, C.byref(params), C.c_void_p(d_sum), C.c_void_p(d_sum_sq),
                                                  C.c_void_p(d_count)))

    def train(self, steps: int) -> float:
        loss = C.c_double()
        check(load().muon_gpu_guide_train(self._h, steps, C.byref(loss)))
        return loss.value

    def forward(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32)
        out = np.zeros((len(f), 64), dtype=np.float32)
        check(load().muon_gpu_guide_forward(self._h, f.ctypes.data_as(C.POINTER(C.c_float)), len(f),
                                            out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def sample(self, features: np.ndarray, u: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Directions (n x 3) drawn from the mixture at each feature row with
        uniforms u (n x 3), and their mixture densities (n)."""
        f = np.ascontiguousarray(features, dtype=np.float32)
        uu = np.ascontiguousarray(u, dtype=np.float32)
        dirs = np.zeros((len(f), 3), dtype=np.float32)
        pdf = np.zeros(len(f), dtype=np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        check(load().muon_gpu_guide_sample(self._h, fp(f), fp(uu), len(f), fp(dirs), fp(pdf)))
        return dirs, pdf

    def gradients(self, features: np.ndarray, dirs: np.ndarray, weights: np.ndarray) -> tuple[np.ndarray, float]:
        f = np.ascontiguousarray(features, dtype=np.float32)
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        w = np.ascontiguousarray(weights, dtype=np.float32)
        g = np.zeros(native.GUIDE_PARAMS, dtype=np.float32)
        loss = C.c_double()
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        check(load().muon_gpu_guide_gradients(self._h, fp(f), fp(d), fp(w), len(f), fp(g), C.byref(loss)))
        return g, loss.value

    def params(self) -> np.ndarray:
        out = np.zeros(native.GUIDE_PARAMS, dtype=np.float32)
        check(load().muon_gpu_guide_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_params(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float32)
        check(load().muon_gpu_guide_set_params(self._h, v.ctypes.data_as(C.POINTER(C.c_float))))

    def set_status(self, status: int) -> None:
        """Writes the device wait-status word (1: as a timed-out tensor-core
        wait leaves it; 0: cleared)."""
        check(load().muon_gpu_guide_set_status(self._h, status))

    def samples(self) -> int:
        n = C.c_uint64()
        check(load().muon_gpu_guide_samples(self._h, C.byref(n)))
        return n.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().muon_gpu_guide_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_file(path: str, **overrides) -> tuple[FilmResult, float]:
    """Parses and renders a scene file; returns the film and the file's gamma."""
    scene = Scene.from_file(path)
    try:
        return scene.render(**overrides), scene.gamma
    finally:
        scene.close()
