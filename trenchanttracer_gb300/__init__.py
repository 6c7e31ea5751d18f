"""GB300-native path-tracing core with the reference's scene formats, compact SBVH layout and
intersect() semantics, backed by libtt.so (include/tt.h)."""
from ._lib import TTError, lib
from .core import (Batch, BVHCompact, Cache, DeviceBVH, Renderer, Scene, camera_meta, hits_to_numpy, make_camera_meta,
                   ray_order_keys, render_meta, render_params)

__all__ = ["TTError", "lib", "Batch", "Cache", "Scene", "BVHCompact", "DeviceBVH", "Renderer", "camera_meta", "make_camera_meta",
           "render_meta", "render_params", "hits_to_numpy", "ray_order_keys"]
