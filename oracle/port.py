"""Python access to the oracle's CPU restatement of the reference renderer.

Test infrastructure: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py, as the checker. See oracle/muon_oracle.cc for
what it restates.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        l = C.CDLL(path)
        l.oracle_last_error.restype = C.c_char_p
        l.oracle_scene_info.argtypes = [C.c_char_p, C.POINTER(C.c_int32)]
        l.oracle_render.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_int,
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_float),
                                    C.POINTER(C.c_uint64)]
        l.oracle_intersect.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_longlong,
                                       C.POINTER(C.c_double)]
        l.oracle_camera_rays.argtypes = [C.c_char_p, C.POINTER(C.c_float)]
        l.oracle_scene_load.restype = C.c_void_p
        l.oracle_scene_load.argtypes = [C.c_char_p, C.c_int]
        l.oracle_scene_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_longlong, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        l.oracle_scene_free.argtypes = [C.c_void_p]
        l.oracle_tonemap.argtypes = [C.POINTER(C.c_float), C.c_longlong, C.c_int, C.c_float, C.POINTER(C.c_uint8)]
        _lib = l
    return _lib


def _check(rc: int) -> None:
    if rc:
        raise RuntimeError(f"oracle error {rc}: {lib().oracle_last_error().decode()}")


@dataclass
class OracleFilm:
    sum: np.ndarray
    sum_sq: np.ndarray
    count: np.ndarray
    film32: np.ndarray      # the reference's FP32 accumulator
    counters: dict

    def mean(self) -> np.ndarray:
        return self.sum / self.count[..., None]


def scene_info(text: str) -> tuple[int, int, int, int]:
    out = (C.c_int32 * 4)()
    _check(lib().oracle_scene_info(text.encode(), out))
    return tuple(out)


def render(text: str, spp: int = 0, seed: int = -1, threads: int = 1, precision: int = 32,
           linear: bool = False) -> OracleFilm:
    """Renders a scene text with the reference algorithm on `threads` host threads."""
    w, h, file_spp, _ = scene_info(text)
    n = spp if spp > 0 else file_spp
    s = np.zeros((h, w, 3))
    q = np.zeros((h, w, 3))
    f32 = np.zeros((h, w, 3), dtype=np.float32)
    cnt = (C.c_uint64 * 8)()
    _check(lib().oracle_render(text.encode(), precision, threads, spp, seed, int(linear),
                               s.ctypes.data_as(C.POINTER(C.c_double)), q.ctypes.data_as(C.POINTER(C.c_double)),
                               f32.ctypes.data_as(C.POINTER(C.c_float)), cnt))
    names = ["primary", "secondary", "object_tests", "object_hits", "bounds_tests", "bounds_hits", "build_ns",
             "render_ns"]
    return OracleFilm(s, q, np.full((h, w), n, dtype=np.uint32), f32, dict(zip(names, list(cnt))))


def tonemap(film32: np.ndarray, spp: int, gamma: float) -> np.ndarray:
    """Film::WriteOutput (muon/film.cc:21-43) on the FP32 accumulator."""
    f = np.ascontiguousarray(film32, dtype=np.float32)
    out = np.zeros(f.shape, dtype=np.uint8)
    lib().oracle_tonemap(f.ctypes.data_as(C.POINTER(C.c_float)), f.size, spp, gamma,
                         out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def intersect(text: str, rays: np.ndarray, precision: int = 32, linear: bool = True):
    """Closest hits for rays (n x 6); returns (distance, prim_id, position, normal)."""
    r = np.ascontiguousarray(rays, dtype=np.float32)
    out = np.zeros((len(r), 8))
    _check(lib().oracle_intersect(text.encode(), precision, int(linear), r.ctypes.data_as(C.POINTER(C.c_float)),
                                  len(r), out.ctypes.data_as(C.POINTER(C.c_double))))
    return out[:, 0], out[:, 1].astype(np.int64), out[:, 2:5], out[:, 5:8]


def camera_rays(text: str) -> np.ndarray:
    w, h, _, _ = scene_info(text)
    rays = np.zeros((h * w, 6), dtype=np.float32)
    _check(lib().oracle_camera_rays(text.encode(), rays.ctypes.data_as(C.POINTER(C.c_float))))
    return rays


class LoadedScene:
    """A scene parsed and built once by the oracle, rendered many times (FP32,
    the reference's precision): for timing the reference algorithm without
    re-parsing a large scene per run."""

    def __init__(self, text: str, linear: bool = False):
        self.width, self.height, self.spp, _ = scene_info(text)
        self._h = lib().oracle_scene_load(text.encode(), int(linear))
        if not self._h:
            raise RuntimeError(f"oracle error: {lib().oracle_last_error().decode()}")

    def render(self, spp: int = 0, seed: int = -1, threads: int = 1, film: bool = False) -> dict:
        """Renders; returns the counters (render_ns: the render alone) and,
        with film=True, the FP64 sums under "sum" / "sum_sq"."""
        cnt = (C.c_uint64 * 8)()
        s = q = None
        if film:
            s = np.zeros((self.height, self.width, 3))
            q = np.zeros((self.height, self.width, 3))
        dp = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))
        _check(lib().oracle_scene_render(self._h, threads, spp, seed, dp(s), dp(q), cnt))
        names = ["primary", "secondary", "object_tests", "object_hits", "bounds_tests", "bounds_hits", "build_ns",
                 "render_ns"]
        out = dict(zip(names, list(cnt)))
        if film:
            out["sum"], out["sum_sq"] = s, q
        return out

    def close(self) -> None:
        if self._h:
            lib().oracle_scene_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
