"""Camera and frame metadata against the reference's own host code (tests/golden/camera_golden.json,
written by the reference's Camera(config) + setFovx(45) + getCameraMeta() and WangHash::encode)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import refhost
from trenchanttracer_gb300 import Scene, _lib, camera_meta, render_meta

ROOT = Path(__file__).resolve().parents[1]


def test_camera_meta_matches_reference(golden_dir, golden_scene_files):
    gold = json.loads((golden_dir / "camera_golden.json").read_text())
    for name, cfg in golden_scene_files.items():
        cm = camera_meta(Scene.load_json(cfg), 45.0)
        got = np.array(list(cm.position) + list(cm.view) + list(cm.up) + list(cm.fov) + [cm.aperture, cm.focal],
                       np.float32)
        want = np.array(gold[name], np.float32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name


def test_wang_hash_and_render_meta(golden_dir):
    gold = json.loads((golden_dir / "camera_golden.json").read_text())["wang_hash"]
    for a, v in gold.items():
        assert _lib.lib().tt_wang_hash(int(a)) == v
    rm = render_meta(5, 16)
    assert rm.hashed_frame == gold.get("5", _lib.lib().tt_wang_hash(5))
    assert np.float32(rm.pi) == np.float32(3.14156265) and rm.samples == 16


_REFERENCE_CAMERAS = r"""
import sys, json, numpy as np
from oracle import refhost
out = [refhost.camera_meta(cfg, float(fx)).tolist() for cfg, fx in json.loads(sys.argv[1])]
print(json.dumps(out))
"""


@pytest.mark.skipif(not refhost.available(), reason="the reference's host code is not built on this host")
def test_random_cameras_match_reference(tmp_path):
    """300 random camera blocks (any key may be left to its default; numbers as long decimals,
    exponents or integers, read as double then rounded to float as the reference's JSON library
    does) and field-of-view angles give the reference's CameraMeta bit for bit. The reference runs
    in a child process."""
    (tmp_path / "m.obj").write_text("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0 1\nvn 0 0 1\n"
                                    "g g\nusemtl a\nf 1/1/1 2/1/2 3/1/3\n")
    (tmp_path / "m.mtl").write_text(json.dumps({"a": {"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}}))
    rng = np.random.default_rng(77)

    def number(lo, hi):
        k = int(rng.integers(4))
        x = float(rng.uniform(lo, hi))
        if k == 0:
            return x
        if k == 1:
            return float("%.3g" % x)
        if k == 2:
            return int(round(x))
        return x * 1e-6

    cases = []
    for k in range(300):
        cam = {"width": int(rng.integers(1, 4097)), "height": int(rng.integers(1, 4097))}
        for key, lo, hi in [("yaw", -7.0, 7.0), ("pitch", -1.5, 1.5), ("focal", 0.1, 20.0), ("aperture", 0.0, 0.5)]:
            if rng.random() < 0.8:
                cam[key] = number(lo, hi)
        if rng.random() < 0.8:
            cam["position"] = [number(-50.0, 50.0) for _ in range(3)]
        cfg = {"work-dir": str(tmp_path), "samples": 1, "material-file": str(tmp_path / "m.mtl"), "hdr-file-name": "",
               "bvh-reload": True, "material-reload": True, "camera": cam,
               "objects": [{"type": "Mesh", "file": str(tmp_path / "m.obj")}]}
        p = tmp_path / f"c{k}.json"
        p.write_text(json.dumps(cfg))
        cases.append((str(p), float(np.float32(rng.uniform(5.0, 150.0)))))
    pr = subprocess.run([sys.executable, "-c", _REFERENCE_CAMERAS, json.dumps(cases)], capture_output=True, text=True,
                        timeout=600, cwd=ROOT, env={**os.environ, "PYTHONPATH": str(ROOT)})
    assert pr.returncode == 0, pr.stderr[-2000:]
    want = json.loads(pr.stdout.strip().splitlines()[-1])
    for (cfg, fx), w in zip(cases, want):
        cm = camera_meta(Scene.load_json(cfg), fx)
        got = np.array(list(cm.position) + list(cm.view) + list(cm.up) + list(cm.fov) + [cm.aperture, cm.focal],
                       np.float32)
        assert np.array_equal(got.view(np.uint32), np.array(w, np.float32).view(np.uint32)), (cfg, got, w)


@pytest.mark.skipif(not refhost.available(), reason="the reference's host code is not built on this host")
def test_wang_hash_matches_reference_on_random_words():
    rng = np.random.default_rng(5)
    for a in list(rng.integers(0, 2**32, 20000, dtype=np.uint64)) + [0, 1, 2**31 - 1, 2**31, 2**32 - 1]:
        assert _lib.lib().tt_wang_hash(int(a)) == refhost.wang_hash(int(a)), int(a)
