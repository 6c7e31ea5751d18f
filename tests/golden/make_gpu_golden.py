"""Generates tests/golden/trace_gpu_golden.npz from the reference's OWN kernel on a GPU.

Runs the reference's intersect() (oracle/_ref/ref_intersect.cubin, prebuilt by
oracle/build_ref.py from the reference sources) on seeded scenes and ray sets and stores, per
set, 4096 rays with the kernel's hit id, distance, material index and interpolated normal for
closest and any hit. The incoherent ray sets are spawned from the reference kernel's own first
hits. Run on a GPU host from the repository root: python tests/golden/make_gpu_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import refgpu  # noqa: E402
from trenchanttracer_gb300 import BVHCompact, Scene, scenes  # noqa: E402

KEEP = 4096


def ray_sets(kind: str, arr: dict):
    if kind == "cornell":
        prim = scenes.pinhole_rays(256, 256, [0.0, 0.0, 1.6], [0.0, 0.0, 0.0], 0.45)
        scale = 1.0
    else:
        scale = 8.0
        cam = scenes.terrain_camera(scale)
        prim = scenes.pinhole_rays(384, 384, cam["eye"], cam["target"], cam["tan_half_fov"])
    yield "primary", prim
    first = refgpu.intersect(arr, prim, True)
    sec, _ = scenes.secondary_rays(prim, first["t"], first["normal"], prim.shape[0], 11, 1e-4 * scale)
    yield "diffuse", sec
    if kind == "terrain":
        yield "shadow", scenes.shadow_rays(prim, first["t"], [-2.0, 32.0, -2.0], prim.shape[0], 13, 1e-4 * scale)
    lo = np.array([-1.2, -0.6, -1.2], np.float32) * scale
    yield "random", scenes.random_rays(prim.shape[0], 5, lo, -lo)


def main() -> None:
    refgpu.build()
    assert refgpu.available(), "the reference cubin or its loader is missing"
    out = {}
    for kind, builder, args in [("cornell", "cornell", [5]), ("terrain", "terrain", [128, 8.0])]:
        mesh = getattr(scenes, builder)(*args)
        arr = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, 8).arrays()
        for set_name, rays in ray_sets(kind, arr):
            name = f"{kind}_{set_name}"
            sub = np.ascontiguousarray(rays[:: max(1, rays.shape[0] // KEEP)][:KEEP])
            out[f"{name}__builder"] = np.array(builder)
            out[f"{name}__args"] = np.array(json.dumps(args))
            out[f"{name}__rays"] = sub
            for closest in (True, False):
                r = refgpu.intersect(arr, sub, closest)
                key = f"{name}__{'closest' if closest else 'any'}"
                for k in ["id", "t", "mat", "normal"]:
                    out[f"{key}_{k}"] = r[k]
            print(name, "hit fraction", float((out[f"{name}__closest_id"] >= 0).mean()), flush=True)
    dst = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent / "trace_gpu_golden.npz"
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    main()
