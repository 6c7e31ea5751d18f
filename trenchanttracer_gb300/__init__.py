"""GB300-native path-tracing core with the reference's scene formats, compact SBVH layout and
intersect() semantics, backed by libtt.so (include/tt.h)."""
from ._lib import TTError, lib
from .core import BVHCompact, DeviceBVH, Scene, hits_to_numpy

__all__ = ["TTError", "lib", "Scene", "BVHCompact", "DeviceBVH", "hits_to_numpy"]
