"""RGBE (.hdr) decoding: this project's loader against the reference's HDRLoader
(src/loader/HDRLoader.cpp:5-152) on pictures in every scanline coding it reads. The reference's
decoded floats are pinned as sha256 hashes in tests/golden/rgbe_golden.json (made by
tests/golden/make_rgbe_golden.py from the reference's own loader); where that loader is built here
the two are also compared directly."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import refhost
from tests.golden.rgbe_files import truncated, write_all
from trenchanttracer_gb300 import Scene

GOLDEN = json.loads((Path(__file__).parent / "golden" / "rgbe_golden.json").read_text())


def _load(tmp_path: Path, hdr: Path) -> np.ndarray:
    cfg = {"work-dir": str(tmp_path), "samples": 1, "material-file": str(tmp_path / "m.mtl"),
           "hdr-file-name": str(hdr), "bvh-reload": True, "material-reload": True,
           "camera": {"width": 8, "height": 8, "position": [0.0, 0.0, 0.0], "yaw": 0.0, "pitch": 0.0,
                      "focal": 1.0, "aperture": 0.0},
           "objects": [{"type": "Mesh", "file": str(tmp_path / "t.obj")}]}
    (tmp_path / "t.obj").write_text("mtllib m.mtl\nusemtl a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0 1\n"
                                    "vn 0 0 1\nf 1/1/1 2/1/2 3/1/3\n")
    (tmp_path / "m.mtl").write_text(json.dumps({"a": {"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}}))
    (tmp_path / "s.json").write_text(json.dumps(cfg))
    return Scene.load_json(tmp_path / "s.json").env()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_rgbe_codings_match_reference_loader(tmp_path, name):
    files = write_all(tmp_path)
    img = _load(tmp_path, files[name])
    g = GOLDEN[name]
    assert list(img.shape) == g["shape"]
    assert hashlib.sha256(np.ascontiguousarray(img, np.float32).tobytes()).hexdigest() == g["sha256"]
    if refhost.available():
        assert np.array_equal(img.view(np.uint32), refhost.load_hdr(str(files[name])).view(np.uint32))


def test_truncated_rgbe_keeps_the_complete_rows(tmp_path):
    path, rows = truncated(tmp_path)
    img = _load(tmp_path, path)
    assert img.shape == (5, 32, 3)
    e = rows[..., 3].astype(np.int32) - 128
    want = (rows[..., :3].astype(np.float32) / 256.0) * np.ldexp(np.float32(1.0), e)[..., None].astype(np.float32)
    assert np.array_equal(img[:3], want.astype(np.float32))
    assert not img[3:].any()  # the scanline the data ends in, and the rows after it, stay zero


@pytest.mark.skipif(not refhost.available(), reason="the reference's loader is not built on this host")
def test_random_rgbe_pictures_match_reference_loader(tmp_path):
    """60 random pictures, 1-400 pixels wide and 1-12 rows high, each row in a coding drawn at
    random (flat, flat with repeat pixels, adaptive run-length where the width allows it), decode
    to the reference loader's floats bit for bit."""
    from tests.golden import rgbe_files as rf
    rng = np.random.default_rng(31)
    for k in range(60):
        w, h = int(rng.integers(1, 401)), int(rng.integers(1, 13))
        rows = []
        for row in rf._pixels(rng, w, h):
            c = int(rng.integers(3))
            if c == 0 and 8 <= w < 32768:
                rows.append(rf._rle_row(rng, row))
            elif c == 1 and w > 3:
                rows.append(rf._flat_row_with_repeats(rng, row))
            else:
                rows.append(rf._flat_row(row))
        p = tmp_path / f"r{k}.hdr"
        p.write_bytes(rf.HEADER + f"-Y {h} +X {w}\n".encode() + b"".join(rows))
        img = _load(tmp_path, p)
        assert np.array_equal(img.view(np.uint32), refhost.load_hdr(str(p)).view(np.uint32)), (k, w, h)
