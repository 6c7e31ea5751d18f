"""The seeded scenes and ray sets behind the golden fixtures, written in the reference's own
file formats (scene JSON, OBJ with `vn` per `v`, material JSON) so that the reference's loader and
this project's loader read the very same files."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from trenchanttracer_gb300 import scenes

LEAF_MAX = [0x7FFFFFF, 8]  # the reference default (SAHHelper.h:80) and the configs' leaf <= 8


def _ico(subdiv: int) -> scenes.Mesh:
    v, t = scenes.icosphere(subdiv)
    return scenes.Mesh(v, v.copy(), t, t.copy(), np.zeros(len(t), np.uint32),
                       [{"name": "sphere", "type": "Diff", "diffuseColor": [0.8, 0.8, 0.8]}])


def _write_mesh(d: Path, name: str, mesh: scenes.Mesh) -> str:
    (d / f"{name}.mtl").write_text(json.dumps(scenes.material_json(mesh.materials)))
    scenes.write_obj(str(d / f"{name}.obj"), mesh, f"{name}.mtl")
    return str(d / f"{name}.obj")


def _config(d: Path, name: str, objects: list, width: int = 64, height: int = 48) -> Path:
    (d / "master.mtl").write_text(json.dumps({
        "white": {"type": "Diff", "diffuseColor": [0.73, 0.73, 0.73]},
        "light": {"type": "Diff", "diffuseColor": [0.0, 0.0, 0.0], "emission": [17.0, 12.0, 4.0]},
        "mirror": {"type": "Spec", "color": [0.9, 0.9, 0.9]},
    }))
    cfg = {"work-dir": str(d), "samples": 1, "material-file": str(d / "master.mtl"), "hdr-file-name": "",
           "bvh-reload": True, "material-reload": True,
           "camera": {"width": width, "height": height, "position": [0.0, 0.1, 0.0], "yaw": 0.3, "pitch": 0.2,
                      "focal": 3.0, "aperture": 0.0},
           "objects": objects}
    p = d / f"{name}.json"
    p.write_text(json.dumps(cfg))
    return p


def write_all(d: Path) -> dict[str, Path]:
    d.mkdir(parents=True, exist_ok=True)
    out = {}
    obj = _write_mesh(d, "ico3", _ico(3))
    out["ico3"] = _config(d, "ico3", [{"type": "Mesh", "file": obj, "transform": {"scale": [8, 8, 8]}}])
    obj = _write_mesh(d, "terrain64", scenes.terrain(64, 0.5))
    out["terrain64"] = _config(d, "terrain64", [{"type": "Mesh", "file": obj, "transform": {"scale": [8, 8, 8]}}])
    obj = _write_mesh(d, "cornell4", scenes.cornell(4))
    out["cornell4"] = _config(d, "cornell4", [{"type": "Mesh", "file": obj,
                                               "transform": {"scale": [2, 2, 2], "translate": [0.0, 0.25, 0.0]}}])
    a = _write_mesh(d, "ico2", _ico(2))
    b = _write_mesh(d, "terrain16", scenes.terrain(16, 0.5, seed=3))
    out["mixed"] = _config(d, "mixed", [
        {"type": "Plane", "p0": [-3, -1, -3], "p1": [-3, -1, 3], "p2": [3, -1, -3], "material": "white"},
        {"type": "Mesh", "file": a, "transform": {"scale": [1.5, 1.5, 1.5], "translate": [0.5, 0.0, 0.0],
                                                  "orientation": [10.0, 90.0, 0.0]}},
        {"type": "Sphere", "radius": 0.5, "position": [1.0, 0.5, 0.0], "material": "mirror"},
        {"type": "Mesh", "file": b, "transform": {"scale": [4, 4, 4], "translate": [0.0, -0.2, 0.0]}},
    ])
    return out


def golden_rays(name: str, cache: np.ndarray, count: int = 6000) -> np.ndarray:
    """Hashed rays around the scene bounds plus axis-aligned rays (zero direction components
    take the 2^-80 guard of the inverse direction) and rays starting inside the scene."""
    hdr = cache[:28].view(np.uint32)
    off = 28 + 16 * int(hdr[0])
    verts = cache[off:off + 16 * int(hdr[3])].view(np.float32).reshape(-1, 4)
    real = verts[verts[:, 0:1].view(np.uint32)[:, 0] != 0x80000000][:, :3]
    lo, hi = real.min(0), real.max(0)
    ext = hi - lo
    seed = sum(map(ord, name))
    outside = scenes.random_rays(count // 2, seed, lo - 0.7 * ext, hi + 0.7 * ext)
    inside = scenes.random_rays(count // 4, seed + 1, lo + 0.25 * ext, hi - 0.25 * ext, tmin=1e-3)
    k = count - outside.shape[0] - inside.shape[0]
    axis = scenes.random_rays(k, seed + 2, lo - 0.2 * ext, hi + 0.2 * ext)
    dirs = np.zeros((k, 3), np.float32)
    comp = np.arange(k) % 6
    dirs[np.arange(k), comp % 3] = np.where(comp < 3, -1.0, 1.0)
    axis[:, 3:6] = dirs
    return np.concatenate([outside, inside, axis]).astype(np.float32)
