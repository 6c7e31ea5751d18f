"""Camera and frame metadata against the reference's own host code (tests/golden/camera_golden.json,
written by the reference's Camera(config) + setFovx(45) + getCameraMeta() and WangHash::encode)."""
import json

import numpy as np

from trenchanttracer_gb300 import Scene, _lib, camera_meta, render_meta


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
