"""ctypes view of include/muon_gpu.h and the loader for libmuon_gpu.so.

The library is built in-tree by muon_gb300/build.py. There is no fallback: if
the shared library cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmuon_gpu.so")
HEADER = os.path.join(HERE, "..", "include", "muon_gpu.h")

MUON_OK = 0
ERRORS = {1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "device timeout", 5: "parse error", 6: "I/O error"}

INTEGRATORS = {"normals": 0, "albedo": 1, "depth": 2, "raytracer": 3, "analyticdirect": 4, "pathtracer": 5}
NEE = {"off": 0, "on": 1, "mis": 2}
IMPORTANCE = {"hemisphere": 0, "cosine": 1, "brdf": 2}
ISECT_FAST, ISECT_WATERTIGHT, ISECT_EXACT = 0, 1, 2
ACCEL_LINEAR, ACCEL_BVH = 0, 1
# MUON_BUILDER_*: host binned SAH, device linear BVH ("gpu"), device binned SAH
BUILDER = {"host": 0, "gpu": 1, "gpu_lbvh": 1, "gpu_sah": 2}  # Scene also takes "auto"
PARTITION = {"uniform": 0, "midpoint": 1, "sah": 2}
RENDER_STATS, RENDER_ACCUMULATE, RENDER_TIMING, RENDER_NO_GRAPH = 1, 2, 4, 8
NOALLOC_SCRATCH_BYTES = 64 << 20


class TransformDesc(C.Structure):
    _fields_ = [("object_to_world", C.c_float * 16), ("world_to_object", C.c_float * 16),
                ("normal_to_world", C.c_float * 16)]


class MaterialDesc(C.Structure):
    _fields_ = [("ambient", C.c_float * 3), ("diffuse", C.c_float * 3), ("specular", C.c_float * 3),
                ("emission", C.c_float * 3), ("shininess", C.c_float), ("roughness", C.c_float),
                ("brdf", C.c_int32), ("pad", C.c_int32)]


class LightDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("color", C.c_float * 3), ("p0", C.c_float * 3), ("p1", C.c_float * 3),
                ("p2", C.c_float * 3)]


class TriangleDesc(C.Structure):
    _fields_ = [("v", (C.c_float * 3) * 3), ("n", (C.c_float * 3) * 3), ("transform", C.c_int32),
                ("material", C.c_int32), ("light", C.c_int32), ("smooth", C.c_int32), ("prim_id", C.c_int32),
                ("pad", C.c_int32)]


class SphereDesc(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("transform", C.c_int32),
                ("material", C.c_int32), ("prim_id", C.c_int32), ("pad", C.c_int32)]


class CameraDesc(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("look_at", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_y_degrees", C.c_float), ("width", C.c_int32), ("height", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("camera", CameraDesc),
                ("transforms", C.POINTER(TransformDesc)), ("num_transforms", C.c_int32),
                ("materials", C.POINTER(MaterialDesc)), ("num_materials", C.c_int32),
                ("lights", C.POINTER(LightDesc)), ("num_lights", C.c_int32),
                ("triangles", C.POINTER(TriangleDesc)), ("num_triangles", C.c_int64),
                ("spheres", C.POINTER(SphereDesc)), ("num_spheres", C.c_int64),
                ("acceleration", C.c_int32), ("partition_strategy", C.c_int32), ("max_leaf_size", C.c_int32),
                ("builder", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("pixel_samples", C.c_int32), ("light_samples", C.c_int32),
                ("light_stratify", C.c_int32), ("next_event_estimation", C.c_int32),
                ("russian_roulette", C.c_int32), ("importance_sampling", C.c_int32), ("min_depth", C.c_int32),
                ("max_depth", C.c_int32), ("sample_offset", C.c_int32), ("seed", C.c_uint64),
                ("intersect_mode", C.c_int32), ("wave_paths", C.c_int32), ("flags", C.c_uint32),
                ("pad", C.c_int32)]


class Film(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("sum", C.POINTER(C.c_double)),
                ("sum_sq", C.POINTER(C.c_double)), ("count", C.POINTER(C.c_uint32))]


class Ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("direction", C.c_float * 3)]


class Hit(C.Structure):
    _fields_ = [("distance", C.c_float), ("prim_id", C.c_int32), ("position", C.c_float * 3),
                ("normal", C.c_float * 3)]


class Stats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("secondary_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("object_tests", C.c_uint64), ("object_hits", C.c_uint64), ("bounds_tests", C.c_uint64),
                ("bounds_hits", C.c_uint64), ("paths", C.c_uint64), ("render_ms", C.c_double),
                ("extend_ms", C.c_double), ("occlude_ms", C.c_double), ("shade_ms", C.c_double),
                ("fold_ms", C.c_double),
                ("kernel_launches", C.c_uint64), ("bvh_nodes", C.c_uint64), ("primitives", C.c_uint64),
                ("extend_rays", C.c_uint64), ("extend_launches", C.c_uint64), ("extend_box_tests", C.c_uint64),
                ("extend_prim_tests", C.c_uint64), ("occlude_rays", C.c_uint64), ("occlude_launches", C.c_uint64),
                ("occlude_box_tests", C.c_uint64), ("occlude_prim_tests", C.c_uint64)]


class BatchSceneStats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("done_ms", C.c_double)]


class BatchTuning(C.Structure):
    _fields_ = [("wave_paths", C.c_int32), ("traversal_blocks_per_sm", C.c_int32), ("candidates", C.c_int32),
                ("pad", C.c_int32), ("best_ms", C.c_double)]


class WalkCounts(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("box_tests", C.c_uint64), ("prim_tests", C.c_uint64), ("hits", C.c_uint64)]


class TraversalProbe(C.Structure):
    _fields_ = [("extend_walked", WalkCounts), ("occlude_walked", WalkCounts), ("extend_rays", C.c_uint64),
                ("occlude_rays", C.c_uint64), ("extend_box_tests", C.c_double), ("extend_prim_tests", C.c_double),
                ("occlude_box_tests", C.c_double), ("occlude_prim_tests", C.c_double)]


class BvhInfo(C.Structure):
    _fields_ = [("nodes", C.c_int64), ("slots", C.c_int64), ("leaves", C.c_int64), ("max_depth", C.c_int32),
                ("max_leaf", C.c_int32)]


class GuideConfig(C.Structure):
    _fields_ = [("batch", C.c_int32), ("wave_paths", C.c_int32), ("record_bounces", C.c_int32),
                ("pool_capacity", C.c_int32), ("learning_rate", C.c_float), ("mixture_fraction", C.c_float),
                ("targets", C.c_int32), ("reserved", C.c_int32), ("seed", C.c_uint64)]


GUIDE_DIRECT, GUIDE_ALL = 0, 1


GUIDE_PARAMS = 33088

# Every entry point declared in include/muon_gpu.h: name -> (restype, argtypes)
SIGNATURES = {
    "muon_parse_scene_file": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "muon_parse_scene_string": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "muon_parsed_scene_desc": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(RenderParams)]),
    "muon_parsed_scene_gamma": (C.c_float, [C.c_void_p]),
    "muon_parsed_scene_output": (C.c_char_p, [C.c_void_p]),
    "muon_parsed_scene_warnings": (C.c_int32, [C.c_void_p]),
    "muon_parsed_scene_free": (None, [C.c_void_p]),
    "muon_film_tonemap": (C.c_int, [C.POINTER(Film), C.c_float, C.POINTER(C.c_uint8)]),
    "muon_film_write": (C.c_int, [C.POINTER(Film), C.c_float, C.c_char_p]),
    "muon_gpu_scene_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    "muon_gpu_scene_destroy": (None, [C.c_void_p]),
    "muon_gpu_release_cached": (None, []),
    "muon_gpu_render": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(Film)]),
    "muon_gpu_render_device": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p,
                                         C.c_void_p]),
    "muon_gpu_render_noalloc": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    "muon_gpu_intersect": (C.c_int, [C.c_void_p, C.POINTER(Ray), C.c_int64, C.c_int32, C.POINTER(Hit)]),
    "muon_gpu_occluded": (C.c_int, [C.c_void_p, C.POINTER(Ray), C.POINTER(C.c_float), C.c_int64, C.c_int32,
                                    C.POINTER(C.c_uint8)]),
    "muon_gpu_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "muon_walk_rays": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(Ray), C.POINTER(C.c_float), C.c_int64, C.c_int32,
                                 C.c_int32, C.POINTER(C.c_int32), C.POINTER(WalkCounts)]),
    "muon_gpu_probe_traversal": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_int32,
                                           C.POINTER(TraversalProbe)]),
    "muon_gpu_measure_read_bandwidth": (C.c_int, [C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_double)]),
    "muon_gpu_scene_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "muon_gpu_scene_bvh": (C.c_int, [C.c_void_p, C.POINTER(BvhInfo), C.c_void_p, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_uint8)]),
    "muon_gpu_last_error": (C.c_char_p, []),
    "muon_gpu_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]),
    "muon_gpu_batch_destroy": (None, [C.c_void_p]),
    "muon_gpu_batch_render_device": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(C.c_void_p),
                                               C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "muon_gpu_batch_render": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(Film)]),
    "muon_gpu_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.POINTER(BatchTuning)]),
    "muon_gpu_batch_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats), C.POINTER(BatchSceneStats)]),
    "muon_gpu_render_batch": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(RenderParams), C.c_int32,
                                        C.POINTER(Film)]),
    "muon_gpu_guide_create": (C.c_int, [C.c_void_p, C.POINTER(GuideConfig), C.POINTER(C.c_void_p)]),
    "muon_gpu_guide_destroy": (None, [C.c_void_p]),
    "muon_gpu_guide_render_device": (C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p, C.c_void_p,
                                               C.c_void_p]),
    "muon_gpu_guide_train": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "muon_gpu_guide_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float)]),
    "muon_gpu_guide_sample": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                         C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "muon_gpu_guide_gradients": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_float),
                                           C.POINTER(C.c_double)]),
    "muon_gpu_guide_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "muon_gpu_guide_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "muon_gpu_guide_samples": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "muon_gpu_guide_set_status": (C.c_int, [C.c_void_p, C.c_int32]),
}

_lib = None


def load() -> C.CDLL:
    """Loads libmuon_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with muon_gb300.build.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class MuonError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


def check(code: int) -> None:
    if code != MUON_OK:
        msg = load().muon_gpu_last_error()
        raise MuonError(code, msg.decode() if msg else "")
