"""ctypes binding of libtt.so (the C ABI declared in include/tt.h).

The library is built in-tree by trenchanttracer_gb300.build; importing this module never
falls back to anything else: if libtt.so is missing the import fails loudly.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libtt.so"

TT_OK = 0
STATUS_NAMES = {0: "TT_OK", 1: "TT_ERR_INVALID", 2: "TT_ERR_IO", 3: "TT_ERR_CUDA", 4: "TT_ERR_TIMEOUT",
                5: "TT_ERR_BOUNDS", 6: "TT_ERR_OOM", 7: "TT_ERR_FORMAT", 8: "TT_ERR_NO_DEVICE"}


class TTError(RuntimeError):
    """A libtt call returned a non-zero tt_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class BvhHeader(C.Structure):
    _fields_ = [("nodes", C.c_uint32), ("tri_count", C.c_uint32), ("leaf_count", C.c_uint32),
                ("vertices", C.c_uint32), ("normals", C.c_uint32), ("tri_indices", C.c_uint32),
                ("mat_indices", C.c_uint32)]


class CameraMeta(C.Structure):
    """tt_camera_meta == the reference's CameraMeta (include/core/Camera.h:8-16)."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("position", C.c_float * 3), ("view", C.c_float * 3),
                ("up", C.c_float * 3), ("fov", C.c_float * 2), ("aperture", C.c_float), ("focal", C.c_float)]


class RenderMeta(C.Structure):
    """tt_render_meta == the reference's RenderMeta (include/core/Renderer.h:24-31)."""
    _fields_ = [("frame_number", C.c_int32), ("hashed_frame", C.c_uint32), ("samples", C.c_int32),
                ("pi", C.c_float), ("two_pi", C.c_float)]


class Material(C.Structure):
    """tt_material (include/tt.h)."""
    _fields_ = [("kind", C.c_int32), ("emission", C.c_float * 3), ("color", C.c_float * 3), ("color2", C.c_float * 3),
                ("roughness", C.c_float), ("ior", C.c_float), ("pad", C.c_float * 4)]


class Geometry(C.Structure):
    """tt_geometry (include/tt.h)."""
    _fields_ = [("kind", C.c_int32), ("material", C.c_int32), ("radius", C.c_float), ("pad", C.c_float),
                ("p0", C.c_float * 3), ("p1", C.c_float * 3), ("p2", C.c_float * 3), ("pad2", C.c_float * 3)]


class RenderParams(C.Structure):
    """tt_render_params (include/tt.h)."""
    _fields_ = [("spp", C.c_int32), ("sample_offset", C.c_int32), ("max_depth", C.c_int32), ("rr_depth", C.c_int32),
                ("seed", C.c_uint32), ("env_scale", C.c_float), ("ray_eps", C.c_float), ("flags", C.c_int32)]


RENDER_ACCUM_F64 = 1
RENDER_NO_ENV_SAMPLING = 2


class LaunchShape(C.Structure):
    """tt_launch_shape (include/tt.h)."""
    _fields_ = [("block", C.c_int32), ("stack_shared", C.c_int32), ("wave_paths", C.c_int32), ("ordered", C.c_int32),
                ("streamed", C.c_int32), ("ms", C.c_float)]

    def as_tuple(self) -> tuple:
        return (self.block, self.stack_shared, self.wave_paths, self.ordered, self.streamed)


class CacheParams(C.Structure):
    """tt_cache_params (include/tt.h)."""
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("ema", C.c_float), ("batch", C.c_int32), ("steps", C.c_int32), ("train_paths", C.c_int32),
                ("spread_c", C.c_float), ("seed", C.c_uint32), ("use_ema", C.c_int32),
                ("bbox_lo", C.c_float * 3), ("bbox_hi", C.c_float * 3), ("mma_kind", C.c_int32),
                ("wait_limit", C.c_int32)]


class View(C.Structure):
    """tt_view (include/tt.h): one view of a batched render."""
    _fields_ = [("cam", CameraMeta), ("spp", C.c_int32), ("sample_offset", C.c_int32), ("seed", C.c_uint32),
                ("reserved", C.c_int32)]

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
F32 = C.c_float
SIGNATURES = {
    "tt_last_error_string": (C.c_char_p, []),
    "tt_version": (C.c_char_p, []),
    "tt_scene_load_json": (I32, [C.c_char_p, C.POINTER(P)]),
    "tt_scene_create": (I32, [P, I32, P, I32, P, P, P, I32, C.POINTER(P)]),
    "tt_scene_counts": (I32, [P, C.POINTER(I32)]),
    "tt_scene_arrays": (I32, [P, P, P, P, P, P]),
    "tt_scene_env": (I32, [P, C.POINTER(I32), C.POINTER(I32), P]),
    "tt_scene_set_env": (I32, [P, I32, I32, P]),
    "tt_scene_materials": (I32, [P, P]),
    "tt_scene_set_materials": (I32, [P, P, I32]),
    "tt_scene_geometries": (I32, [P, P]),
    "tt_scene_set_geometries": (I32, [P, P, I32]),
    "tt_scene_free": (None, [P]),
    "tt_bvh_build": (I32, [P, F32, I32, I32, I32, C.POINTER(P)]),
    "tt_bvh_save": (I32, [P, C.c_char_p]),
    "tt_bvh_load": (I32, [C.c_char_p, C.POINTER(P)]),
    "tt_bvh_header_get": (I32, [P, C.POINTER(BvhHeader)]),
    "tt_bvh_arrays": (I32, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "tt_bvh_free": (None, [P]),
    "tt_bvh_upload": (I32, [P, C.POINTER(P)]),
    "tt_dbvh_free": (None, [P]),
    "tt_dbvh_set_variant": (I32, [P, I32]),
    "tt_dbvh_set_l2_window": (I32, [P, I64]),
    "tt_dbvh_get_variant": (I32, [P, C.POINTER(I32)]),
    "tt_dbvh_autotune": (I32, [P, P, I64, P, I32, I32, P, P]),
    "tt_trace": (I32, [P, P, I64, P, I32, P]),
    "tt_trace_ext": (I32, [P, P, I64, P, I32, P]),
    "tt_trace_host": (I32, [P, P, I64, P, I32, P]),
    "tt_ray_order_keys": (I32, [P, I64, P, P, P, P]),
    "tt_ray_order_keys_device": (I32, [P, I64, P, P, P, P, P]),
    "tt_dbvh_check": (I32, [P, P]),
    "tt_trace_host_noalloc": (I32, [P, P, P, P, I64, P, I32, P]),
    "tt_camera_meta_from_scene": (I32, [P, F32, C.POINTER(CameraMeta)]),
    "tt_render_meta_init": (I32, [I32, I32, C.POINTER(RenderMeta)]),
    "tt_wang_hash": (C.c_uint32, [C.c_uint32]),
    "tt_renderer_create": (I32, [P, P, C.POINTER(P)]),
    "tt_renderer_free": (None, [P]),
    "tt_render_compat": (I32, [P, C.POINTER(CameraMeta), C.POINTER(RenderMeta), P, P]),
    "tt_renderer_check": (I32, [P, P]),
    "tt_compat_replay": (I32, [P, C.POINTER(CameraMeta), C.POINTER(RenderMeta), P, I64, P, P]),
    "tt_native_sample_probe": (I32, [P, I32, P, I64, P]),
    "tt_render_params_default": (I32, [C.POINTER(RenderParams)]),
    "tt_render_native": (I32, [P, C.POINTER(CameraMeta), C.POINTER(RenderParams), P, P]),
    "tt_renderer_env_tables": (I32, [P, P, P]),
    "tt_renderer_set_launch": (I32, [P, C.POINTER(LaunchShape)]),
    "tt_renderer_get_launch": (I32, [P, C.POINTER(LaunchShape)]),
    "tt_renderer_stats": (I32, [P, P, I32]),
    "tt_renderer_launches": (I32, [P, P, I32]),
    "tt_batch_create": (I32, [P, P, I32, C.POINTER(RenderParams), C.POINTER(P)]),
    "tt_batch_info": (I32, [P, C.POINTER(I64), C.POINTER(I64)]),
    "tt_batch_render": (I32, [P, P, I32, P]),
    "tt_batch_graph_kernels": (I32, [P, C.POINTER(I32)]),
    "tt_batch_autotune": (I32, [P, I64, P, P, I32, C.POINTER(I32)]),
    "tt_batch_free": (I32, [P]),
    "tt_cache_params_default": (I32, [C.POINTER(CacheParams)]),
    "tt_cache_create": (I32, [C.POINTER(CacheParams), C.POINTER(P)]),
    "tt_cache_free": (I32, [P]),
    "tt_cache_param_count": (I32, [C.POINTER(I32)]),
    "tt_cache_get_weights": (I32, [P, P, I32]),
    "tt_cache_set_weights": (I32, [P, P]),
    "tt_cache_encode": (I32, [P, P, I64, P, P]),
    "tt_cache_infer": (I32, [P, P, I64, P, I32, P]),
    "tt_cache_gradient": (I32, [P, P, P, I64, P, P, P]),
    "tt_cache_train": (I32, [P, P, P, I64, I32, P, P]),
    "tt_cache_steps": (I32, [P, C.POINTER(I32)]),
    "tt_cache_check": (I32, [P, P]),
    "tt_render_cached": (I32, [P, P, C.POINTER(CameraMeta), C.POINTER(RenderParams), P, I32, P]),
}

_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Loads libtt.so once and declares every exported signature."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(status: int) -> None:
    if status != TT_OK:
        msg = lib().tt_last_error_string()
        # the message may quote bytes of a malformed input file
        raise TTError(status, msg.decode(errors="replace") if msg else "")
