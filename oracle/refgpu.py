"""The reference's own device intersect() on the GPU (oracle/_ref/ref_intersect.cubin through
oracle/ref/ref_gpu_loader.cpp).

Test infrastructure only: the device oracle that pins hit ids and distances bit for bit, and the
reference GPU baseline. `available()` is False without a GPU or without the prebuilt cubin.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "ref" / "ref_gpu_loader.cpp"
LIB = HERE / "_build" / "libref_gpu.so"
CUBIN = HERE / "_ref" / "ref_intersect.cubin"
_h = None


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cuda = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + str(cuda / "include"), str(SRC), "-o", str(tmp),
           "-L" + str(cuda / "lib64"), "-L" + str(cuda / "lib64" / "stubs"), "-lcudart_static", "-lcuda",
           "-lpthread", "-ldl", "-lrt"]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("ref_gpu_loader build failed:\n" + proc.stdout)
    tmp.replace(LIB)
    return LIB


def available() -> bool:
    return CUBIN.exists() and LIB.exists()


def _load():
    global _h
    if _h is None:
        h = C.CDLL(str(LIB))
        h.ref_gpu_error.restype = C.c_char_p
        h.ref_gpu_trace.restype = C.c_int
        h.ref_gpu_trace.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        _h = h
    return _h


RENDER_CUBIN = HERE / "_ref" / "ref_render.cubin"


def render_available() -> bool:
    return RENDER_CUBIN.exists() and LIB.exists()


def _render_args(bvh_arrays: dict, materials: list, geometries: list, env: np.ndarray | None, cam) -> tuple:
    """The scene as the flat arrays ref_gpu_render takes (kept alive by the returned tuple)."""
    a = {k: np.ascontiguousarray(bvh_arrays[k]) for k in ["nodes", "vertices", "normals", "tri_indices",
                                                         "mat_indices"]}
    geo = np.zeros((max(1, len(geometries)), 16), np.float32)
    geo_mat = np.zeros(max(1, len(geometries)), np.int32)
    for i, g in enumerate(geometries):
        geo[i, 0] = g.kind
        geo[i, 1:4] = list(g.p0)
        geo[i, 4:7] = list(g.p1)
        geo[i, 7:10] = list(g.p2)
        geo[i, 10] = g.radius
        geo_mat[i] = g.material
    mat = np.zeros((max(1, len(materials)), 16), np.float32)
    for i, m in enumerate(materials):
        mat[i, 0] = m.kind
        mat[i, 1:4] = list(m.emission)
        mat[i, 4:7] = list(m.color)
        mat[i, 7:10] = list(m.color2)
    if env is None:
        env_a, ew, eh = np.zeros(3, np.float32), 0, 0
    else:
        env_a = np.ascontiguousarray(env, dtype=np.float32)
        eh, ew = env_a.shape[0], env_a.shape[1]
    cam13 = np.array(list(cam.position) + list(cam.view) + list(cam.up) + list(cam.fov) + [cam.aperture, cam.focal],
                     np.float32)
    keep = (a, geo, geo_mat, mat, env_a, cam13)
    args = (a["nodes"].ctypes.data, a["nodes"].shape[0], a["vertices"].ctypes.data, a["vertices"].shape[0],
            a["normals"].ctypes.data, a["tri_indices"].ctypes.data, a["mat_indices"].ctypes.data, geo.ctypes.data,
            geo_mat.ctypes.data, len(geometries), mat.ctypes.data, len(materials), env_a.ctypes.data, ew, eh,
            cam13.ctypes.data, cam.width, cam.height)
    return keep, args


_SCENE_ARGTYPES = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                   C.c_int, C.c_int, C.c_int, C.c_uint, C.c_int, C.c_float, C.c_float, C.c_void_p]


LANE_VOTE_CUBIN = HERE / "_ref" / "ref_render_lane_vote.cubin"


def render(bvh_arrays: dict, materials: list, geometries: list, env: np.ndarray | None, cam, meta,
           accum: np.ndarray, lane_vote: bool = False) -> tuple[np.ndarray, float]:
    """One frame of the reference's own pathTracingKernel. materials / geometries: the
    tt_material / tt_geometry records of the scene; cam / meta: CameraMeta / RenderMeta;
    accum: (W*H*3,) float32 starting contents. lane_vote: the build whose intersect() stops
    looking for leaves per lane instead of per warp (ref_render_lane_vote.cubin). Returns
    (accumulation buffer, kernel ms)."""
    h = _load()
    if not hasattr(h, "_render_ready"):
        h.ref_gpu_render.restype = C.c_int
        h.ref_gpu_render.argtypes = _SCENE_ARGTYPES + [C.c_void_p]
        h._render_ready = True
    keep, args = _render_args(bvh_arrays, materials, geometries, env, cam)
    out = np.ascontiguousarray(accum, dtype=np.float32).copy()
    ms = C.c_float(0.0)
    rc = h.ref_gpu_render(str(LANE_VOTE_CUBIN if lane_vote else RENDER_CUBIN).encode(), *args, meta.frame_number, meta.hashed_frame, meta.samples,
                          meta.pi, meta.two_pi, out.ctypes.data, C.byref(ms))
    del keep
    if rc != 0:
        raise RuntimeError("reference GPU render failed: " + h.ref_gpu_error().decode())
    return out, float(ms.value)


PROBE_CUBIN = HERE / "_ref" / "ref_render_probe.cubin"


def probe_available() -> bool:
    return PROBE_CUBIN.exists() and LIB.exists()


def render_probe(bvh_arrays: dict, materials: list, geometries: list, env: np.ndarray | None, cam, meta,
                 accum: np.ndarray, capacity: int) -> tuple[np.ndarray, np.ndarray, int]:
    """One frame of the reference's pathTracingKernel built with recording samplers
    (ref_render_probe.cu): every material interaction is recorded (field 0 of a record is the
    reference's MaterialType: DIFF, METAL, SPEC, REFR, COAT). Returns (accumulation buffer, the
    first records as a (m, 64) uint32 array, m <= capacity, the number of interactions the frame
    made)."""
    h = _load()
    if not hasattr(h, "_probe_ready"):
        h.ref_gpu_render_probe.restype = C.c_int
        h.ref_gpu_render_probe.argtypes = _SCENE_ARGTYPES + [C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
        h._probe_ready = True
    keep, args = _render_args(bvh_arrays, materials, geometries, env, cam)
    out = np.ascontiguousarray(accum, dtype=np.float32).copy()
    recs = np.zeros((max(1, capacity), 64), np.uint32)
    made = C.c_uint64(0)
    rc = h.ref_gpu_render_probe(str(PROBE_CUBIN).encode(), *args, meta.frame_number, meta.hashed_frame, meta.samples,
                                meta.pi, meta.two_pi, out.ctypes.data, recs.ctypes.data, capacity, C.byref(made))
    del keep
    if rc != 0:
        raise RuntimeError("reference GPU probe render failed: " + h.ref_gpu_error().decode())
    kept = made.value if made.value <= capacity else capacity - 1
    return out, recs[:kept], int(made.value)


def intersect(bvh_arrays: dict, rays: np.ndarray, closest: bool, reps: int = 1) -> dict:
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    n = rays.shape[0]
    a = {k: np.ascontiguousarray(bvh_arrays[k]) for k in ["nodes", "vertices", "normals", "tri_indices",
                                                         "mat_indices"]}
    out = {"id": np.empty(n, np.int32), "mat": np.empty(n, np.int32), "t": np.empty(n, np.float32),
           "normal": np.empty((n, 3), np.float32)}
    ms = C.c_float(0.0)
    rc = _load().ref_gpu_trace(str(CUBIN).encode(), a["nodes"].ctypes.data, a["nodes"].shape[0],
                               a["vertices"].ctypes.data, a["vertices"].shape[0], a["normals"].ctypes.data,
                               a["tri_indices"].ctypes.data, a["mat_indices"].ctypes.data, rays.ctypes.data, n,
                               int(closest), out["id"].ctypes.data, out["mat"].ctypes.data, out["t"].ctypes.data,
                               out["normal"].ctypes.data, reps, C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference GPU intersect failed: " + _load().ref_gpu_error().decode())
    out["ms"] = float(ms.value)
    return out
