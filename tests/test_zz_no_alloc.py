"""The allocation-free host-buffer entry point, tt_trace_host_noalloc.

Some callers cannot allocate device memory (an application that owns all device memory through
its own arena, or a frame loop that must not stall on a cudaMalloc); they upload the BVH into
their own memory and trace through this entry point, which stages rays and hits in a fixed array
inside libtt.so. This file is collected last so that a failure here does not hide any other test.
"""
import ctypes as C

import numpy as np
import pytest

from trenchanttracer_gb300 import BVHCompact, DeviceBVH, Scene, _lib, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_RAYS = 1 << 18  # TT_NOALLOC_MAX_RAYS in include/tt.h


def _noalloc(arrays_dev, rays: np.ndarray, closest: bool) -> np.ndarray:
    hits = np.full((rays.shape[0], 2), -7, np.int32)
    nodes, verts, tri = arrays_dev
    st = _lib.lib().tt_trace_host_noalloc(C.c_void_p(nodes.data_ptr()), C.c_void_p(verts.data_ptr()),
                                          C.c_void_p(tri.data_ptr()), C.c_void_p(rays.ctypes.data), rays.shape[0],
                                          C.c_void_p(hits.ctypes.data), int(closest), None)
    _lib.check(st)
    return hits


def test_noalloc_matches_host_entry_point_on_consecutive_calls():
    torch.cuda.init()
    mesh = scenes.terrain(96, 8.0, seed=5)
    bvh = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, 8)
    a = bvh.arrays()
    # the caller's own device copies of the BVH arrays (allocated by the caller, not by libtt)
    dev = (torch.from_numpy(a["nodes"]).cuda(), torch.from_numpy(a["vertices"]).cuda(),
           torch.from_numpy(a["tri_indices"]).cuda())
    dbvh = DeviceBVH(bvh)
    cam = scenes.terrain_camera(8.0)
    first = scenes.pinhole_rays(256, 200, cam["eye"], cam["target"], cam["tan_half_fov"])
    second = scenes.random_rays(MAX_RAYS, 3, [-9.0, -2.0, -9.0], [9.0, 4.0, 9.0])
    for rays, closest in [(first, True), (second, True), (first, False)]:
        want = np.empty((rays.shape[0], 2), np.int32)
        dbvh.intersect_host(rays, want, closest=closest)
        got = _noalloc(dev, rays, closest)
        assert np.array_equal(got, want), "tt_trace_host_noalloc differs from tt_trace_host"
    assert (_noalloc(dev, first, True)[:, 0] >= 0).mean() > 0.5


def test_noalloc_rejects_oversized_batches():
    rays = np.zeros((MAX_RAYS + 1, 8), np.float32)
    hits = np.zeros((MAX_RAYS + 1, 2), np.int32)
    st = _lib.lib().tt_trace_host_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                          C.c_void_p(rays.ctypes.data), rays.shape[0], C.c_void_p(hits.ctypes.data),
                                          1, None)
    assert st == 1  # TT_ERR_INVALID
    assert b"staging capacity" in _lib.lib().tt_last_error_string()
