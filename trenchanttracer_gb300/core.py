"""Python mirror of the reference's scene / BVH / traversal interfaces over libtt.so.

Names follow the reference's classes: ``Scene`` (core/Scene.h), ``BVHCompact``
(bvh/BVHCompact.h: build, ``save``, load from ``bvh.cache``) and ``DeviceBVH`` holding the
device arrays that intersect() reads. ``DeviceBVH.intersect`` is intersect(ray, bvh,
needClosestHit) (include/geometry/IntersectKernel.cuh:78) over a whole batch of rays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check, lib

RAY_DTYPE = np.float32  # a ray is 8 float32: origin xyz, direction xyz, tmin, tmax


def _ptr(a: np.ndarray | None) -> C.c_void_p:
    return C.c_void_p(0 if a is None else a.ctypes.data)


class Scene:
    """Triangle soup + materials (reference core/Scene.h)."""

    def __init__(self, handle: C.c_void_p, materials: list | None = None):
        self._h = handle
        self.materials = materials or []

    @classmethod
    def load_json(cls, path: str | os.PathLike) -> "Scene":
        """Config + SceneLoader::load: the reference's scene JSON / OBJ / material / .hdr."""
        h = C.c_void_p()
        check(lib().tt_scene_load_json(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, vertices, normals, vidx, nidx=None, mat=None, materials=None) -> "Scene":
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        vi = np.ascontiguousarray(vidx, dtype=np.int32).reshape(-1, 3)
        ni = vi if nidx is None else np.ascontiguousarray(nidx, dtype=np.int32).reshape(-1, 3)
        m = None if mat is None else np.ascontiguousarray(mat, dtype=np.uint32).reshape(-1)
        h = C.c_void_p()
        check(lib().tt_scene_create(_ptr(v), v.shape[0], _ptr(n), n.shape[0], _ptr(vi), _ptr(ni), _ptr(m),
                                    vi.shape[0], C.byref(h)))
        return cls(h, materials)

    @classmethod
    def from_mesh(cls, mesh) -> "Scene":
        sc = cls.from_arrays(mesh.vertices, mesh.normals, mesh.vidx, mesh.nidx, mesh.mat, mesh.materials)
        if mesh.materials:
            sc.set_materials(mesh.materials)
        return sc

    MATERIAL_KINDS = {"Diff": 0, "Metal": 1, "Spec": 2, "Refr": 3, "Coat": 4, "GGX": 5, "Dielectric": 6}

    def set_materials(self, materials: list) -> None:
        """Material-JSON style dicts ({"type": "Diff", "diffuseColor": [...], "emission": [...]}, ...)."""
        arr = (_lib.Material * max(1, len(materials)))()
        for m, d in zip(arr, materials):
            m.kind = self.MATERIAL_KINDS[d["type"]]
            m.emission[:] = [float(x) for x in d.get("emission", [0.0, 0.0, 0.0])]
            col = d.get("diffuseColor", d.get("color", d.get("F0", [0.0, 0.0, 0.0])))
            m.color[:] = [float(x) for x in col]
            m.color2[:] = [float(x) for x in d.get("specularColor", [0.0, 0.0, 0.0])]
            m.roughness = float(d.get("roughness", 0.5))
            m.ior = float(d.get("ior", 1.4 if d["type"] == "Refr" else 1.5))
        check(lib().tt_scene_set_materials(self._h, arr, len(materials)))

    def materials_raw(self) -> list:
        n = self.counts()["materials"]
        arr = (_lib.Material * max(1, n))()
        check(lib().tt_scene_materials(self._h, arr))
        return list(arr)[:n]

    def set_geometries(self, geoms: list) -> None:
        """Dicts {"type": "Plane", "p0", "p1", "p2", "material": idx} or {"type": "Sphere", "radius",
        "position", "material": idx}."""
        arr = (_lib.Geometry * max(1, len(geoms)))()
        for g, d in zip(arr, geoms):
            g.kind = 3 if d["type"] == "Plane" else 0
            g.material = int(d["material"])
            if d["type"] == "Plane":
                g.p0[:], g.p1[:], g.p2[:] = ([float(x) for x in d[k]] for k in ("p0", "p1", "p2"))
            else:
                g.radius = float(d["radius"])
                g.p0[:] = [float(x) for x in d["position"]]
        check(lib().tt_scene_set_geometries(self._h, arr, len(geoms)))

    def geometries_raw(self) -> list:
        n = self.counts()["geometries"]
        arr = (_lib.Geometry * max(1, n))()
        check(lib().tt_scene_geometries(self._h, arr))
        return list(arr)[:n]

    def set_env(self, rgb: np.ndarray | None) -> None:
        """(h, w, 3) float32 linear RGB, row 0 first; None removes the environment."""
        if rgb is None:
            check(lib().tt_scene_set_env(self._h, 0, 0, None))
            return
        a = np.ascontiguousarray(rgb, dtype=np.float32)
        check(lib().tt_scene_set_env(self._h, a.shape[1], a.shape[0], _ptr(a)))

    def counts(self) -> dict:
        c = (C.c_int32 * 5)()
        check(lib().tt_scene_counts(self._h, c))
        return dict(zip(["triangles", "vertices", "normals", "materials", "geometries"], list(c)))

    def arrays(self) -> dict:
        c = self.counts()
        out = {"vertices": np.empty((c["vertices"], 3), np.float32),
               "normals": np.empty((c["normals"], 3), np.float32),
               "vidx": np.empty((c["triangles"], 3), np.int32),
               "nidx": np.empty((c["triangles"], 3), np.int32),
               "mat": np.empty(c["triangles"], np.uint32)}
        check(lib().tt_scene_arrays(self._h, *(_ptr(out[k]) for k in ["vertices", "normals", "vidx", "nidx", "mat"])))
        return out

    def env(self) -> np.ndarray | None:
        """The scene's environment map as (h, w, 3) float32, or None."""
        w, h = C.c_int32(), C.c_int32()
        check(lib().tt_scene_env(self._h, C.byref(w), C.byref(h), None))
        if w.value == 0:
            return None
        out = np.empty((h.value, w.value, 3), np.float32)
        check(lib().tt_scene_env(self._h, C.byref(w), C.byref(h), _ptr(out)))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tt_scene_free(self._h)
            self._h = None


class BVHCompact:
    """Host-side compact SBVH arrays (reference bvh/BVHCompact.h), built or read from bvh.cache."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @classmethod
    def build(cls, scene: Scene, split_alpha: float = 1e-5, leaf_min: int = 1, leaf_max: int = 0x7FFFFFF,
              threads: int = 0) -> "BVHCompact":
        h = C.c_void_p()
        check(lib().tt_bvh_build(scene._h, split_alpha, leaf_min, leaf_max, threads, C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path: str | os.PathLike) -> "BVHCompact":
        h = C.c_void_p()
        check(lib().tt_bvh_load(os.fsencode(path), C.byref(h)))
        return cls(h)

    def save(self, path: str | os.PathLike) -> None:
        check(lib().tt_bvh_save(self._h, os.fsencode(path)))

    @property
    def header(self) -> dict:
        hd = _lib.BvhHeader()
        check(lib().tt_bvh_header_get(self._h, C.byref(hd)))
        return {f: getattr(hd, f) for f, _ in hd._fields_}

    def arrays(self) -> dict:
        """Copies of the five arrays: nodes/vertices/normals as (n, 4) int32 bit patterns."""
        hd = self.header
        p = [C.c_void_p() for _ in range(5)]
        check(lib().tt_bvh_arrays(self._h, *(C.byref(x) for x in p)))

        def grab(ptr, count, dtype, cols=None):
            n = count * (cols or 1)
            if n == 0:
                return np.zeros((0, cols) if cols else 0, dtype)
            buf = (C.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr.value)
            a = np.frombuffer(buf, dtype=dtype).copy()
            return a.reshape(-1, cols) if cols else a

        return {"nodes": grab(p[0], hd["nodes"], np.int32, 4),
                "vertices": grab(p[1], hd["vertices"], np.int32, 4),
                "normals": grab(p[2], hd["normals"], np.int32, 4),
                "tri_indices": grab(p[3], hd["tri_indices"], np.int32),
                "mat_indices": grab(p[4], hd["mat_indices"], np.uint32)}

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tt_bvh_free(self._h)
            self._h = None


class DeviceBVH:
    """The compact BVH resident on the current CUDA device."""

    def __init__(self, bvh: BVHCompact):
        h = C.c_void_p()
        check(lib().tt_bvh_upload(bvh._h, C.byref(h)))
        self._h = h
        self.header = bvh.header

    def intersect(self, rays, hits, closest: bool = True, stream: int = 0, ext: bool = False) -> None:
        """rays: CUDA tensor (n, 8) float32; hits: CUDA tensor (n, 2) int32 [id, t bits]
        (or (n, 6) for ext = id, mat, t, normal xyz). Launch only; no synchronisation."""
        n = rays.shape[0]
        fn = lib().tt_trace_ext if ext else lib().tt_trace
        check(fn(self._h, C.c_void_p(rays.data_ptr()), n, C.c_void_p(hits.data_ptr()), int(bool(closest)),
                 C.c_void_p(stream)))

    def intersect_host(self, rays: np.ndarray, hits: np.ndarray, closest: bool = True, stream: int = 0) -> None:
        """Host buffers: rays (n, 8) float32, hits (n, 2) int32; synchronous."""
        assert rays.dtype == np.float32 and rays.flags.c_contiguous and hits.flags.c_contiguous
        check(lib().tt_trace_host(self._h, _ptr(rays), rays.shape[0], _ptr(hits), int(bool(closest)),
                                  C.c_void_p(stream)))

    VARIANT_WARP, VARIANT_WARP_SH16, VARIANT_WARP_SH32, VARIANT_DYNAMIC, VARIANT_WARP_VOTE = 0, 1, 2, 3, 4
    VARIANT_SORTED, VARIANT_SH16_OCC, VARIANT_SORTED_OCC = 5, 6, 7
    NUM_VARIANTS = 8
    DETERMINISTIC_VARIANTS = (0, 1, 2, 3, 5, 6, 7)

    def set_l2_window(self, nbytes: int) -> None:
        """Bytes of the node array's top levels kept persisting in L2 (tt_dbvh_set_l2_window)."""
        check(lib().tt_dbvh_set_l2_window(self._h, int(nbytes)))

    def set_variant(self, variant: int) -> None:
        """Kernel shape of the traversal calls (include/tt.h, tt_dbvh_set_variant)."""
        check(lib().tt_dbvh_set_variant(self._h, int(variant)))

    @property
    def variant(self) -> int:
        v = C.c_int32()
        check(lib().tt_dbvh_get_variant(self._h, C.byref(v)))
        return v.value

    def autotune(self, rays, hits, closest: bool = True, include_vote: bool = False, stream: int = 0) -> list:
        """Times every kernel variant on these device rays, keeps the fastest; returns ms per variant."""
        ms = (C.c_float * self.NUM_VARIANTS)()
        check(lib().tt_dbvh_autotune(self._h, C.c_void_p(rays.data_ptr()), rays.shape[0],
                                     C.c_void_p(hits.data_ptr()), int(bool(closest)), int(bool(include_vote)),
                                     C.c_void_p(stream), ms))
        return list(ms)

    def check(self, stream: int = 0) -> None:
        check(lib().tt_dbvh_check(self._h, C.c_void_p(stream)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tt_dbvh_free(self._h)
            self._h = None


def camera_meta(scene: Scene, fovx: float = 45.0) -> _lib.CameraMeta:
    """Camera(config) + setFovx(fovx) + getCameraMeta() for a JSON scene's camera block."""
    cm = _lib.CameraMeta()
    check(lib().tt_camera_meta_from_scene(scene._h, fovx, C.byref(cm)))
    return cm


def make_camera_meta(width: int, height: int, position, view, up=(0.0, 1.0, 0.0), fov=(45.0, 45.0),
                     aperture: float = 0.0, focal: float = 1.0) -> _lib.CameraMeta:
    cm = _lib.CameraMeta()
    cm.width, cm.height = int(width), int(height)
    cm.position[:] = [float(x) for x in position]
    cm.view[:] = [float(x) for x in view]
    cm.up[:] = [float(x) for x in up]
    cm.fov[:] = [float(x) for x in fov]
    cm.aperture, cm.focal = float(aperture), float(focal)
    return cm


def render_meta(frame_number: int, samples: int) -> _lib.RenderMeta:
    rm = _lib.RenderMeta()
    check(lib().tt_render_meta_init(frame_number, samples, C.byref(rm)))
    return rm


class Renderer:
    """The device half of the reference's Renderer (src/core/Renderer.cpp:8-57), without GL."""

    def __init__(self, dbvh: DeviceBVH, scene: Scene):
        h = C.c_void_p()
        check(lib().tt_renderer_create(dbvh._h, scene._h, C.byref(h)))
        self._h = h
        self._keep = (dbvh, scene)

    def render_compat(self, cam: _lib.CameraMeta, meta: _lib.RenderMeta, accum, stream: int = 0) -> None:
        """One frame of the reference's path tracer into accum (CUDA tensor, W*H*3 float32)."""
        check(lib().tt_render_compat(self._h, C.byref(cam), C.byref(meta), C.c_void_p(accum.data_ptr()),
                                     C.c_void_p(stream)))

    def compat_replay(self, cam: _lib.CameraMeta, meta: _lib.RenderMeta, records_in, records_out,
                      stream: int = 0) -> None:
        """Re-runs recorded material interactions, environment lookups and primary rays (CUDA
        int32 tensors of shape (n, 64), the tt_compat_interaction layout) through tt_render_compat's
        own arithmetic into records_out."""
        if records_in.shape != records_out.shape or records_in.shape[-1] != 64:
            raise ValueError("records must be (n, 64) 32-bit words, in and out of the same shape")
        check(lib().tt_compat_replay(self._h, C.byref(cam), C.byref(meta), C.c_void_p(records_in.data_ptr()),
                                     int(records_in.shape[0]), C.c_void_p(records_out.data_ptr()),
                                     C.c_void_p(stream)))

    # numpy layout of tt_sample_probe (160 bytes)
    SAMPLE_PROBE_DTYPE = np.dtype([("material", "<i4"), ("entering", "<i4"), ("n", "<f4", 3), ("wo", "<f4", 3),
                                   ("u", "<f4", 3), ("pad0", "<i4"), ("pcg_state", "<u8"), ("pcg_seq", "<u8"),
                                   ("wi", "<f4", 3), ("weight", "<f4", 3), ("pdf", "<f4"), ("eval_pdf", "<f4"),
                                   ("eval", "<f4", 3), ("specular", "<i4"), ("pcg_out", "<u4", 8),
                                   ("texel", "<i4"), ("pad1", "<i4", 3)])
    PROBE_BSDF, PROBE_ENV, PROBE_PCG32 = 0, 1, 2

    def sample_probe(self, what: int, queries: np.ndarray, stream: int = 0) -> np.ndarray:
        """Runs the native renderer's sampling code on host queries (SAMPLE_PROBE_DTYPE records)
        on the GPU and returns the filled records (tt_native_sample_probe)."""
        import torch
        q = np.ascontiguousarray(queries, dtype=self.SAMPLE_PROBE_DTYPE)
        d = torch.from_numpy(q.view(np.uint8).copy()).cuda()
        check(lib().tt_native_sample_probe(self._h, int(what), C.c_void_p(d.data_ptr()), int(q.shape[0]),
                                           C.c_void_p(stream)))
        torch.cuda.synchronize()
        return d.cpu().numpy().view(self.SAMPLE_PROBE_DTYPE).copy()

    def render_native(self, cam: _lib.CameraMeta, params: _lib.RenderParams, accum, stream: int = 0) -> None:
        """Native wavefront path tracer: adds spp samples per pixel to accum (CUDA tensor W*H*3,
        float32, or float64 with the RENDER_ACCUM_F64 flag; row 0 = top)."""
        check(lib().tt_render_native(self._h, C.byref(cam), C.byref(params), C.c_void_p(accum.data_ptr()),
                                     C.c_void_p(stream)))

    def render_cached(self, cache: "Cache", cam: _lib.CameraMeta, params: _lib.RenderParams, accum,
                      train: bool = True, stream: int = 0) -> None:
        """The native path tracer with the learned radiance cache (include/tt.h, tt_render_cached)."""
        check(lib().tt_render_cached(self._h, cache._h, C.byref(cam), C.byref(params), C.c_void_p(accum.data_ptr()),
                                     int(bool(train)), C.c_void_p(stream)))

    def set_launch(self, block: int, stack_shared: int, wave_paths: int, ordered: int = 0, streamed: int = 1) -> None:
        """Launch shape of the native kernels (include/tt.h, tt_launch_shape); ordered = 1 orders
        each extension queue by origin and direction cell before tracing it; streamed = 1 streams
        a render of more paths than one wave through a refilled pool of wave_paths slots."""
        shape = _lib.LaunchShape(int(block), int(stack_shared), int(wave_paths), int(ordered), int(streamed), 0.0)
        check(lib().tt_renderer_set_launch(self._h, C.byref(shape)))

    @property
    def launch(self) -> tuple:
        shape = _lib.LaunchShape()
        check(lib().tt_renderer_get_launch(self._h, C.byref(shape)))
        return shape.as_tuple()

    def stats(self, reset: bool = False) -> dict:
        """Rays and paths the native path tracer traced since the last reset (synchronous)."""
        out = np.zeros(3, np.uint64)
        check(lib().tt_renderer_stats(self._h, _ptr(out), int(bool(reset))))
        return {"extension_rays": int(out[0]), "shadow_rays": int(out[1]), "paths": int(out[2])}

    def launches(self, reset: bool = False) -> int:
        """Path-tracer kernels issued since the last reset (include/tt.h, tt_renderer_launches)."""
        out = np.zeros(1, np.uint64)
        check(lib().tt_renderer_launches(self._h, _ptr(out), int(bool(reset))))
        return int(out[0])

    def env_tables(self, env_w: int, env_h: int) -> tuple[np.ndarray, np.ndarray]:
        marg = np.empty(env_h + 1, np.float32)
        cond = np.empty((env_h, env_w + 1), np.float32)
        check(lib().tt_renderer_env_tables(self._h, _ptr(marg), _ptr(cond)))
        return marg, cond

    def check(self, stream: int = 0) -> None:
        check(lib().tt_renderer_check(self._h, C.c_void_p(stream)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tt_renderer_free(self._h)
            self._h = None


class Batch:
    """Many views of any size and sample count in one graph-captured wavefront render
    (include/tt.h, tt_batch_*). views: sequence of (CameraMeta, spp, sample_offset, seed)."""

    def __init__(self, renderer: Renderer, views, params: _lib.RenderParams):
        arr = (_lib.View * len(views))()
        for k, (cam, spp, offset, seed) in enumerate(views):
            arr[k].cam = cam
            arr[k].spp, arr[k].sample_offset, arr[k].seed = int(spp), int(offset), int(seed)
        h = C.c_void_p()
        check(lib().tt_batch_create(renderer._h, arr, len(views), C.byref(params), C.byref(h)))
        self._h = h
        self._keep = renderer
        self.sizes = [(int(v.cam.width), int(v.cam.height)) for v in arr]
        tp, ae = C.c_int64(), C.c_int64()
        check(lib().tt_batch_info(self._h, C.byref(tp), C.byref(ae)))
        self.total_paths, self.accum_elems = tp.value, ae.value

    def render(self, accum, use_graph: bool = True, stream: int = 0) -> None:
        """Adds every view's samples to accum (CUDA tensor of accum_elems floats / doubles)."""
        assert accum.numel() >= self.accum_elems
        check(lib().tt_batch_render(self._h, C.c_void_p(accum.data_ptr()), int(bool(use_graph)), C.c_void_p(stream)))

    @property
    def graph_kernels(self) -> int:
        n = C.c_int32()
        check(lib().tt_batch_graph_kernels(self._h, C.byref(n)))
        return n.value

    def autotune(self, sample_paths: int = 0, stream: int = 0) -> list:
        """Times launch shapes on the batch's first paths (include/tt.h, tt_batch_autotune), keeps
        the fastest; returns [(block, stack_shared, wave_paths, ordered, streamed, ms)]."""
        res = (_lib.LaunchShape * 64)()
        n = C.c_int32()
        check(lib().tt_batch_autotune(self._h, int(sample_paths), C.c_void_p(stream), res, 64, C.byref(n)))
        return [r.as_tuple() + (r.ms,) for r in res[:min(n.value, 64)]]

    def split(self, accum) -> list:
        """The per-view (H, W, 3) images of an accumulation buffer (torch tensor or numpy array)."""
        out, off = [], 0
        for w, h in self.sizes:
            out.append(accum[off:off + 3 * w * h].reshape(h, w, 3))
            off += 3 * w * h
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tt_batch_free(self._h)
            self._h = None


class Cache:
    """The learned radiance cache (include/tt.h, tt_cache_*). Tensors are CUDA torch tensors:
    records (n, 16) float32, targets (n, 3) float32."""

    def __init__(self, bbox_lo, bbox_hi, **kw):
        p = _lib.CacheParams()
        check(lib().tt_cache_params_default(C.byref(p)))
        p.bbox_lo[:] = [float(x) for x in bbox_lo]
        p.bbox_hi[:] = [float(x) for x in bbox_hi]
        for k, v in kw.items():
            setattr(p, k, v)
        h = C.c_void_p()
        check(lib().tt_cache_create(C.byref(p), C.byref(h)))
        self._h = h
        self.params = p
        n = C.c_int32()
        check(lib().tt_cache_param_count(C.byref(n)))
        self.num_params = n.value

    def weights(self, which: int = 0) -> np.ndarray:
        """0: master weights, 1: averaged weights, 2: last gradient (compact [out][in] per layer)."""
        w = np.empty(self.num_params, np.float32)
        check(lib().tt_cache_get_weights(self._h, _ptr(w), int(which)))
        return w

    def set_weights(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.num_params
        check(lib().tt_cache_set_weights(self._h, _ptr(w)))

    def encode(self, rec):
        import torch
        out = torch.empty((rec.shape[0], 160), dtype=torch.bfloat16, device=rec.device)
        check(lib().tt_cache_encode(self._h, C.c_void_p(rec.data_ptr()), rec.shape[0], C.c_void_p(out.data_ptr()),
                                    None))
        return out

    def infer(self, rec, use_ema: bool = False):
        import torch
        out = torch.empty((rec.shape[0], 3), dtype=torch.float32, device=rec.device)
        check(lib().tt_cache_infer(self._h, C.c_void_p(rec.data_ptr()), rec.shape[0], C.c_void_p(out.data_ptr()),
                                   int(bool(use_ema)), None))
        return out

    def gradient(self, rec, target) -> tuple[np.ndarray, float]:
        g = np.empty(self.num_params, np.float32)
        loss = C.c_float()
        check(lib().tt_cache_gradient(self._h, C.c_void_p(rec.data_ptr()), C.c_void_p(target.data_ptr()),
                                      rec.shape[0], _ptr(g), C.byref(loss), None))
        return g, loss.value

    def train(self, rec, target, steps: int = 1) -> float:
        loss = C.c_float()
        check(lib().tt_cache_train(self._h, C.c_void_p(rec.data_ptr()), C.c_void_p(target.data_ptr()), rec.shape[0],
                                   int(steps), C.byref(loss), None))
        return loss.value

    @property
    def steps(self) -> int:
        n = C.c_int32()
        check(lib().tt_cache_steps(self._h, C.byref(n)))
        return n.value

    def check(self, stream: int = 0) -> None:
        check(lib().tt_cache_check(self._h, C.c_void_p(stream)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().tt_cache_free(self._h)
            self._h = None


def render_params(**kw) -> _lib.RenderParams:
    """tt_render_params with the library defaults, overridden by keyword."""
    p = _lib.RenderParams()
    check(lib().tt_render_params_default(C.byref(p)))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def ray_order_keys(rays: np.ndarray, lo, hi) -> tuple[np.ndarray, int]:
    """The key the ordered trace variants sort rays (n, 8) float32 by, and its width in bits
    (include/tt.h, tt_ray_order_keys)."""
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    assert rays.ndim == 2 and rays.shape[1] == 8
    keys = np.empty(rays.shape[0], np.uint32)
    lo_a = np.ascontiguousarray(lo, dtype=np.float32)
    hi_a = np.ascontiguousarray(hi, dtype=np.float32)
    bits = C.c_int32()
    check(lib().tt_ray_order_keys(_ptr(rays), rays.shape[0], _ptr(lo_a), _ptr(hi_a), _ptr(keys), C.byref(bits)))
    return keys, bits.value


def hits_to_numpy(hits: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(n, 2) int32 [id, t bits] -> (ids int32, t float32)."""
    h = np.ascontiguousarray(hits).view(np.int32).reshape(-1, 2)
    return h[:, 0].copy(), h[:, 1].copy().view(np.float32)
