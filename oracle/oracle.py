"""Build and ctypes access for the oracle's C restatement (oracle/tt_oracle.c).

ORACLE — test infrastructure. Used only by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, to check results or as the reported CPU baseline; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "tt_oracle_pt.c"  # includes tt_oracle.c
SBVH_SRC = HERE / "tt_oracle_sbvh.c"
SRCS = [HERE / "tt_oracle.c", SRC, SBVH_SRC]
LIB = HERE / "_build" / "liboracle.so"

SLAB_FMA, CROSS_A, CROSS_B, DOT_A, DOT_B, INTERP_A, INTERP_B = 1, 2, 4, 8, 16, 32, 64
PLAIN = 0
# The contraction nvcc 13.0 applies to the reference's intersect() on sm_103a: x*y - z and
# a*b - c*d fuse the LEFT product, a*b + c*d + e*f fuses the first sum's left product and then
# the last product. Pinned against the reference kernel's own outputs on a GB300
# (tests/golden/trace_gpu_golden.npz, tests/test_oracle_golden.py); of the five candidate
# patterns only this one reproduces every id, distance and normal bit.
DEVICE = SLAB_FMA | CROSS_A | DOT_B | INTERP_B

_h = None


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(s.stat().st_mtime for s in SRCS):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-D_POSIX_C_SOURCE=199309L", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", str(SRC), str(SBVH_SRC), "-o", str(tmp), "-lm"]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stdout)
    tmp.replace(LIB)
    return LIB


def _load():
    global _h
    if _h is None:
        build()
        h = C.CDLL(str(LIB))
        h.oracle_intersect.restype = C.c_int64
        h.oracle_intersect.argtypes = [C.c_void_p] * 5 + [C.c_void_p, C.c_int64, C.c_int, C.c_int] + \
            [C.c_void_p] * 5 + [C.c_int]
        h.oracle_sbvh_build.restype = C.c_int
        h.oracle_sbvh_build.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_float, C.c_int, C.c_int, C.c_char_p,
                                        C.POINTER(C.c_double)]
        h.oracle_max_threads.restype = C.c_int
        h.oracle_wang_hash.restype = C.c_uint32
        h.oracle_wang_hash.argtypes = [C.c_uint32]
        h.oracle_env_tables.restype = None
        h.oracle_env_tables.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        h.oracle_render_native.restype = C.c_int
        h.oracle_render_native.argtypes = [C.c_void_p] * 5 + [C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                                              C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                              C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                                                              C.c_void_p, C.c_int]
        _h = h
    return _h


def env_tables(env: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Marginal (h+1) and conditional (h, w+1) CDFs of an (h, w, 3) environment map."""
    env = np.ascontiguousarray(env, dtype=np.float32)
    h, w = env.shape[:2]
    marg = np.empty(h + 1, np.float32)
    cond = np.empty((h, w + 1), np.float32)
    _load().oracle_env_tables(env.ctypes.data, w, h, marg.ctypes.data, cond.ctypes.data)
    return marg, cond


def render_native(bvh_arrays: dict, materials, geometries, env: np.ndarray | None, cam, params, tanx: float,
                  tany: float, threads: int = 0) -> np.ndarray:
    """The native path tracer restated on the CPU: returns the accumulation buffer (W*H*3 floats)
    of params.spp samples per pixel. materials / geometries: ctypes arrays of tt_material /
    tt_geometry; cam / params: tt_camera_meta / tt_render_params."""
    a = [np.ascontiguousarray(bvh_arrays[k]) for k in ["nodes", "vertices", "normals", "tri_indices", "mat_indices"]]
    if env is None:
        env_a, ew, eh = np.zeros(3, np.float32), 0, 0
        marg, cond = np.zeros(1, np.float32), np.zeros(1, np.float32)
    else:
        env_a = np.ascontiguousarray(env, dtype=np.float32)
        eh, ew = env_a.shape[:2]
        marg, cond = env_tables(env_a)
    accum = np.zeros(3 * cam.width * cam.height, np.float32)
    mats = (C.c_byte * max(1, C.sizeof(materials)))()
    C.memmove(mats, materials, C.sizeof(materials))
    geos = (C.c_byte * max(1, C.sizeof(geometries)))()
    if C.sizeof(geometries):
        C.memmove(geos, geometries, C.sizeof(geometries))
    _load().oracle_render_native(*(x.ctypes.data for x in a), mats, len(materials), geos, len(geometries),
                                 env_a.ctypes.data, ew, eh, marg.ctypes.data, cond.ctypes.data, C.byref(cam),
                                 C.byref(params), tanx, tany, accum.ctypes.data, threads)
    return accum


def intersect(bvh_arrays: dict, rays: np.ndarray, closest: bool, arith: int = DEVICE, counters: bool = False,
              normals: bool = False, threads: int = 0) -> dict:
    """bvh_arrays: the dict of BVHCompact.arrays() (or of a loaded bvh.cache)."""
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    n = rays.shape[0]
    out = {"id": np.empty(n, np.int32), "t": np.empty(n, np.float32), "mat": np.empty(n, np.int32)}
    if normals:
        out["normal"] = np.empty((n, 3), np.float32)
    if counters:
        out["counters"] = np.empty((n, 4), np.uint32)
    a = [np.ascontiguousarray(bvh_arrays[k]) for k in ["nodes", "vertices", "normals", "tri_indices", "mat_indices"]]
    ov = _load().oracle_intersect(*(x.ctypes.data for x in a), rays.ctypes.data, n, int(closest), arith,
                                  out["id"].ctypes.data, out["t"].ctypes.data, out["mat"].ctypes.data,
                                  out["normal"].ctypes.data if normals else None,
                                  out["counters"].ctypes.data if counters else None, threads)
    out["overflow"] = int(ov)
    return out


def sbvh_build(vertices: np.ndarray, normals: np.ndarray, vidx: np.ndarray, nidx: np.ndarray, mat: np.ndarray | None,
               cache_path: str | Path, split_alpha: float = 1e-5, leaf_min: int = 1,
               leaf_max: int = 0x7FFFFFF) -> float:
    """The reference's SBVH build and compact emission restated in C (tt_oracle_sbvh.c), single
    threaded as the reference runs it: writes bvh.cache to cache_path (read it with read_cache)
    and returns the build + emission time in seconds."""
    v = np.ascontiguousarray(vertices, np.float32)
    n = np.ascontiguousarray(normals, np.float32)
    vi = np.ascontiguousarray(vidx, np.int32)
    ni = np.ascontiguousarray(nidx, np.int32)
    m = None if mat is None else np.ascontiguousarray(mat, np.uint32)
    secs = C.c_double(0.0)
    rc = _load().oracle_sbvh_build(v.ctypes.data, v.size // 3, n.ctypes.data, n.size // 3, vi.ctypes.data,
                                   ni.ctypes.data, None if m is None else m.ctypes.data, vi.size // 3,
                                   split_alpha, leaf_min, leaf_max, str(cache_path).encode(), C.byref(secs))
    if rc != 0:
        raise RuntimeError(f"oracle SBVH build failed ({rc})")
    return float(secs.value)


def max_threads() -> int:
    return int(_load().oracle_max_threads())


def wang_hash(a: int) -> int:
    return int(_load().oracle_wang_hash(a))


def read_cache(path: str | Path) -> dict:
    """Reads a bvh.cache (7 x u32 header, then the five arrays) without libtt."""
    raw = np.fromfile(path, dtype=np.uint8)
    hdr = raw[:28].view(np.uint32)
    nodes, tri_count, leaf_count, nv, nn, nt, nm = (int(x) for x in hdr)
    off = 28

    def take(count, dtype, cols=None):
        nonlocal off
        size = count * np.dtype(dtype).itemsize * (cols or 1)
        a = raw[off:off + size].view(dtype)
        off += size
        return a.reshape(-1, cols) if cols else a

    return {"header": {"nodes": nodes, "tri_count": tri_count, "leaf_count": leaf_count, "vertices": nv,
                       "normals": nn, "tri_indices": nt, "mat_indices": nm},
            "nodes": take(nodes, np.int32, 4), "vertices": take(nv, np.int32, 4), "normals": take(nn, np.int32, 4),
            "tri_indices": take(nt, np.int32), "mat_indices": take(nm, np.uint32)}
