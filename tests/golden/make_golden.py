"""Generates the CPU golden fixtures from the reference's OWN code (oracle/_ref/libttref_host.so,
built by oracle/build_ref.py from the reference checkout).

  bvh_golden.json        per seeded scene and leaf setting: sha256 of the bvh.cache written by the
                         reference's SceneLoader + BVH + BVHCompact::save, its header, and the
                         sha256 of the scene arrays its loader produced
  trace_host_golden.npz  per scene and closest/any: rays and the reference intersect() results
                         (compiled for the host: every product and sum rounded separately)
  camera_golden.json     the reference's Camera::getCameraMeta for a few configs, and WangHash
                         values

Run from the repository root: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build_ref, refhost  # noqa: E402
from tests.golden import golden_scenes  # noqa: E402

OUT = Path(__file__).resolve().parent


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def main() -> None:
    build_ref.build()
    assert refhost.available(), "oracle/_ref/libttref_host.so is missing"
    golden = {}
    traces = {}
    cams = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, cfg in golden_scenes.write_all(Path(tmp)).items():
            arrays = refhost.scene_arrays(str(cfg))
            entry = {"scene_sha256": sha(b"".join(np.ascontiguousarray(arrays[k]).tobytes()
                                                  for k in ["vertices", "normals", "vidx", "nidx", "mat"]))}
            for leaf_max in golden_scenes.LEAF_MAX:
                cache = Path(tmp) / f"{name}_{leaf_max}.cache"
                refhost.build_json(str(cfg), str(cache), 1e-5, 1, leaf_max)
                raw = cache.read_bytes()
                hdr = np.frombuffer(raw[:28], np.uint32).tolist()
                entry[str(leaf_max)] = {"sha256": sha(raw), "header": hdr}
                if leaf_max == golden_scenes.LEAF_MAX[-1]:
                    rays = golden_scenes.golden_rays(name, np.frombuffer(raw, np.uint8))
                    traces[f"{name}_rays"] = rays
                    for closest in (1, 0):
                        r = refhost.intersect(str(cache), rays, bool(closest))
                        key = f"{name}_{'closest' if closest else 'any'}"
                        for k in ["id", "t", "mat", "normal"]:
                            traces[f"{key}_{k}"] = r[k]
            golden[name] = entry
            cams[name] = refhost.camera_meta(str(cfg), 45.0).tolist()
    cams["wang_hash"] = {str(a): refhost.wang_hash(a) for a in [0, 1, 2, 3, 7, 100, 12345, 2**31 - 1, 2**32 - 1]}
    (OUT / "bvh_golden.json").write_text(json.dumps(golden, indent=1, sort_keys=True) + "\n")
    (OUT / "camera_golden.json").write_text(json.dumps(cams, indent=1, sort_keys=True) + "\n")
    np.savez_compressed(OUT / "trace_host_golden.npz", **traces)
    print("wrote", sorted(p.name for p in OUT.glob("*golden*")))


if __name__ == "__main__":
    main()
