"""The allocation-free host-buffer entry point, tt_trace_host_noalloc.

Some callers cannot allocate device memory (an application that owns all device memory through
its own arena, or a frame loop that must not stall on a cudaMalloc); they upload the BVH into
their own memory and trace through this entry point, which stages rays and hits in a fixed array
inside libtt.so. This file is collected last so that a failure here does not hide any other test.
"""
import ctypes as C
import struct

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


def _self_loop_arrays(child1_box_empty: bool):
    """A corrupt BVH whose root lists itself as both children (the one the trace tests use):
    child 1 far from every ray makes a ray loop without pushing (the iteration cap), child 1 over
    the rays makes it push until the stack bound."""
    big = 1e3
    c1lo, c1hi = (1e6, 1e6 + 1.0) if child1_box_empty else (-big, big)
    nodes = np.zeros((4, 4), np.float32)
    nodes[0] = [-big, big, -big, big]
    nodes[1] = [c1lo, c1hi, c1lo, c1hi]
    nodes[2] = [-big, big, c1lo, c1hi]
    nodes.view(np.int32)[3] = [0, 0, 0, 0]
    verts = np.array([[0x80000000, 0, 0, 0]], np.uint32).view(np.int32)
    return (torch.from_numpy(nodes.view(np.int32).copy()).cuda(), torch.from_numpy(verts.copy()).cuda(),
            torch.zeros(1, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("child1_empty,status,word", [(True, 4, b"iteration cap"), (False, 5, b"stack")])
def test_noalloc_reports_traversal_errors_then_starts_clean(child1_empty, status, word):
    """The error word lives in the shared array's header: a corrupt BVH's error reaches the
    caller as a status and message, and the next call on a valid BVH starts from a clean word."""
    rays = scenes.random_rays(64, 3, [-1] * 3, [1] * 3)
    hits = np.zeros((64, 2), np.int32)
    bad = _self_loop_arrays(child1_empty)
    st = _lib.lib().tt_trace_host_noalloc(C.c_void_p(bad[0].data_ptr()), C.c_void_p(bad[1].data_ptr()),
                                          C.c_void_p(bad[2].data_ptr()), C.c_void_p(rays.ctypes.data), 64,
                                          C.c_void_p(hits.ctypes.data), 1, None)
    assert st == status  # 4 = TT_ERR_TIMEOUT (iteration cap), 5 = TT_ERR_BOUNDS (stack)
    assert word in _lib.lib().tt_last_error_string()
    mesh = scenes.terrain(32, 8.0, seed=2)
    bvh = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, 8)
    a = bvh.arrays()
    dev = (torch.from_numpy(a["nodes"]).cuda(), torch.from_numpy(a["vertices"]).cuda(),
           torch.from_numpy(a["tri_indices"]).cuda())
    good = scenes.random_rays(4096, 9, [-9.0, -2.0, -9.0], [9.0, 4.0, 9.0])
    want = np.empty((good.shape[0], 2), np.int32)
    DeviceBVH(bvh).intersect_host(good, want, closest=True)
    assert np.array_equal(_noalloc(dev, good, True), want)


def test_noalloc_warm_up_call():
    """n = 0 loads the library's device code on the current device (reserving the staging array)
    and returns TT_OK: what a caller does before its own arena takes the device's memory."""
    torch.cuda.init()
    assert _lib.lib().tt_trace_host_noalloc(None, None, None, None, 0, None, 1, None) == 0
