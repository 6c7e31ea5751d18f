"""ctypes access to oracle/_ref/libttref_host.so: the reference's own scene loader, SBVH builder,
camera and host-compiled intersect() (see oracle/build_ref.py).

Test infrastructure only. The library exists only where the reference checkout was available
to build it; callers skip when `available()` is False.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_ref" / "libttref_host.so"
_h = None


def available() -> bool:
    if not LIB.exists():
        return False
    try:
        _load()
        return True
    except OSError:
        return False  # e.g. an x86 build on an Arm host


def _load():
    global _h
    if _h is None:
        h = C.CDLL(str(LIB))
        h.ref_build_json.restype = C.c_int
        h.ref_build_json.argtypes = [C.c_char_p, C.c_char_p, C.c_float, C.c_int, C.c_int]
        h.ref_scene_arrays.restype = C.c_int
        h.ref_scene_arrays.argtypes = [C.c_char_p, C.POINTER(C.c_int)] + [C.c_void_p] * 5
        h.ref_camera_meta.restype = C.c_int
        h.ref_camera_meta.argtypes = [C.c_char_p, C.c_float, C.c_void_p]
        h.ref_scene_materials.restype = C.c_int
        h.ref_scene_materials.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.c_void_p, C.c_void_p]
        h.ref_wang_hash.restype = C.c_uint
        h.ref_wang_hash.argtypes = [C.c_uint]
        h.ref_load_hdr.restype = C.c_int
        h.ref_load_hdr.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_longlong]
        h.ref_intersect_host.restype = C.c_int
        h.ref_intersect_host.argtypes = [C.c_char_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_int]
        _h = h
    return _h


def build_json(config: str, cache: str, split_alpha: float = 1e-5, leaf_min: int = 1,
               leaf_max: int = 0x7FFFFFF) -> None:
    if _load().ref_build_json(os.fsencode(config), os.fsencode(cache), split_alpha, leaf_min, leaf_max) != 0:
        raise RuntimeError("reference build failed")


def scene_arrays(config: str) -> dict:
    h = _load()
    counts = (C.c_int * 3)()
    if h.ref_scene_arrays(os.fsencode(config), counts, None, None, None, None, None) != 0:
        raise RuntimeError("reference scene load failed")
    t, v, n = counts
    out = {"vertices": np.empty((v, 3), np.float32), "normals": np.empty((n, 3), np.float32),
           "vidx": np.empty((t, 3), np.int32), "nidx": np.empty((t, 3), np.int32), "mat": np.empty(t, np.uint32)}
    h.ref_scene_arrays(os.fsencode(config), counts, *(out[k].ctypes.data for k in
                                                         ["vertices", "normals", "vidx", "nidx", "mat"]))
    return out


def scene_materials(config: str) -> tuple[np.ndarray, np.ndarray]:
    """(materials (m, 10), analytic objects (g, 13)) as ref_scene_materials flattens them."""
    h = _load()
    counts = (C.c_int * 2)()
    if h.ref_scene_materials(os.fsencode(config), counts, None, None) != 0:
        raise RuntimeError("reference scene load failed")
    mats = np.zeros((counts[0], 10), np.float32)
    geoms = np.zeros((counts[1], 13), np.float32)
    h.ref_scene_materials(os.fsencode(config), counts, mats.ctypes.data, geoms.ctypes.data)
    return mats, geoms


def camera_meta(config: str, fovx: float = 45.0) -> np.ndarray:
    out = np.empty(13, np.float32)
    if _load().ref_camera_meta(os.fsencode(config), fovx, out.ctypes.data) != 0:
        raise RuntimeError("reference camera failed")
    return out


def wang_hash(a: int) -> int:
    return int(_load().ref_wang_hash(a))


def intersect(cache: str, rays: np.ndarray, closest: bool, threads: int = 0) -> dict:
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    n = rays.shape[0]
    out = {"id": np.empty(n, np.int32), "mat": np.empty(n, np.int32), "t": np.empty(n, np.float32),
           "normal": np.empty((n, 3), np.float32)}
    rc = _load().ref_intersect_host(os.fsencode(cache), rays.ctypes.data, n, int(closest), out["id"].ctypes.data,
                                    out["mat"].ctypes.data, out["t"].ctypes.data, out["normal"].ctypes.data, threads)
    if rc != 0:
        raise RuntimeError("reference intersect failed")
    return out


def load_hdr(path: str, max_texels: int = 1 << 22) -> np.ndarray:
    """The reference's HDRLoader on an RGBE file: (height, width, 3) float32."""
    buf = np.zeros(3 * max_texels, np.float32)
    w, h = C.c_int(0), C.c_int(0)
    if _load().ref_load_hdr(os.fsencode(path), C.byref(w), C.byref(h), buf.ctypes.data, buf.size) != 0:
        raise RuntimeError(f"reference HDRLoader failed on {path}")
    return buf[:3 * w.value * h.value].reshape(h.value, w.value, 3).copy()
