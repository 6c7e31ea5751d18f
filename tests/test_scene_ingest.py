"""Scene ingest beyond the golden scenes: the chunked parallel OBJ parser gives the same arrays as
the reference's loader and as itself on any number of threads (chunk boundaries fall inside
lines, groups and material switches); OBJs without normals or with fewer normals than vertices
load (the reference rejects or misreads them); mutated scene, OBJ, material and RGBE files load or
fail with an error status, never a crash."""
import hashlib
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import refhost
from trenchanttracer_gb300 import Scene, TTError

ROOT = Path(__file__).resolve().parents[1]


def _tricky_obj(d: Path, with_normals: bool = True, short_normals: bool = False) -> Path:
    rng = np.random.default_rng(5)
    v = rng.uniform(-3, 3, (240, 3)).astype(np.float32)
    n = rng.normal(size=(240, 3))
    n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
    if short_normals:
        n = n[:100]
    lines = ["# tricky obj\r", "mtllib m.mtl\r"]
    for i, p in enumerate(v):
        sep = "\t" if i % 7 == 0 else " "
        lines.append(f"v{sep}{float(p[0])!r} {float(p[1])!r}  {float(p[2])!r}" + ("\r" if i % 3 == 0 else ""))
    if with_normals:
        for q in n:
            lines.append(f"vn {float(q[0])!r} {float(q[1])!r} {float(q[2])!r}")
    mats = ["a", "b", "c"]
    k = 0
    for gi in range(9):
        lines.append(f"g grp{gi}")
        lines.append(f"usemtl {mats[gi % 3]}")
        for _ in range(int(rng.integers(3, 12))):
            deg = int(rng.integers(3, 6))
            idx = rng.choice(240, deg, replace=False)
            if with_normals:
                ni = rng.integers(0, len(n), deg)
                lines.append("f " + " ".join(f"{a + 1}/{(a % 5) + 1}/{b + 1}" for a, b in zip(idx, ni)))
            else:
                lines.append("f " + " ".join(f"{a + 1}" for a in idx))
            k += 1
        if gi == 4:
            lines.append("usemtl c")  # a material switch inside a group
    (d / "m.obj").write_text("\n".join(lines) + "\n")
    (d / "m.mtl").write_text(json.dumps({"a": {"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]},
                                         "b": {"type": "Spec", "color": [0.9, 0.9, 0.9]},
                                         "c": {"type": "Diff", "diffuseColor": [0.2, 0.7, 0.2]}}))
    cfg = {"work-dir": str(d), "samples": 1, "material-file": str(d / "m.mtl"), "hdr-file-name": "",
           "bvh-reload": True, "material-reload": True,
           "camera": {"width": 8, "height": 8, "position": [0.0, 0.0, 0.0], "yaw": 0.0, "pitch": 0.0,
                      "focal": 1.0, "aperture": 0.0},
           "objects": [{"type": "Mesh", "file": str(d / "m.obj"),
                        "transform": {"scale": [2, 3, 4], "orientation": [10, 20, 30], "translate": [1, 2, 3]}}]}
    (d / "s.json").write_text(json.dumps(cfg))
    return d / "s.json"


def _digest(arrays: dict) -> str:
    h = hashlib.sha256()
    for k in ["vertices", "normals", "vidx", "nidx", "mat"]:
        h.update(np.ascontiguousarray(arrays[k]).tobytes())
    return h.hexdigest()


@pytest.mark.skipif(not refhost.available(), reason="the reference's loader is not built on this host")
def test_tricky_obj_matches_reference_loader(tmp_path):
    cfg = _tricky_obj(tmp_path)
    mine = Scene.load_json(cfg).arrays()
    ref = refhost.scene_arrays(str(cfg))
    for k in ["vertices", "normals", "vidx", "nidx", "mat"]:
        assert np.array_equal(np.asarray(mine[k]).view(np.uint32) if mine[k].dtype == np.float32 else mine[k],
                              np.asarray(ref[k]).view(np.uint32) if ref[k].dtype == np.float32 else ref[k]), k


def test_parse_is_independent_of_thread_count(tmp_path):
    cfg = _tricky_obj(tmp_path)
    code = ("import sys, hashlib, numpy as np; sys.path.insert(0, %r); from trenchanttracer_gb300 import Scene; "
            "a = Scene.load_json(%r).arrays(); h = hashlib.sha256(); "
            "[h.update(np.ascontiguousarray(a[k]).tobytes()) for k in ['vertices','normals','vidx','nidx','mat']]; "
            "print(h.hexdigest())") % (str(ROOT), str(cfg))
    digests = set()
    for threads in ("1", "3", "7", "16"):
        env = dict(os.environ, OMP_NUM_THREADS=threads)
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
        digests.add(out.stdout.strip().splitlines()[-1])
    assert len(digests) == 1
    assert digests == {_digest(Scene.load_json(cfg).arrays())}


def test_obj_without_normals_gets_vertex_normals(tmp_path):
    cfg = _tricky_obj(tmp_path, with_normals=False)
    a = Scene.load_json(cfg).arrays()
    assert a["normals"].shape == a["vertices"].shape
    assert np.array_equal(a["nidx"], a["vidx"])
    length = np.linalg.norm(a["normals"], axis=1)
    assert np.allclose(length, 1.0, atol=1e-5)


def test_obj_with_fewer_normals_than_vertices(tmp_path):
    cfg = _tricky_obj(tmp_path, short_normals=True)
    a = Scene.load_json(cfg).arrays()
    assert a["normals"].shape[0] == 100 and a["vertices"].shape[0] == 240
    assert np.allclose(np.linalg.norm(a["normals"], axis=1), 1.0, atol=1e-5)  # all transformed and normalised
    assert a["nidx"].max() < 100


def test_malformed_obj_reports_the_first_error(tmp_path):
    cfg = _tricky_obj(tmp_path)
    obj = tmp_path / "m.obj"
    text = obj.read_text().splitlines()
    text.insert(50, "v 1.0 2.0")  # a short vertex line, early in the file
    text.insert(len(text) - 3, "usemtl nosuch")
    obj.write_text("\n".join(text) + "\n")
    with pytest.raises(TTError) as e:
        Scene.load_json(cfg)
    assert "short v line" in str(e.value)


_MUTATE_AND_LOAD = r"""
import random, shutil, sys
from pathlib import Path
from trenchanttracer_gb300 import Scene, TTError
base, work, seeds = Path(sys.argv[1]), Path(sys.argv[2]), int(sys.argv[3])
names = sorted(p.name for p in base.iterdir())
tokens = [b"-1", b"0", b"99999999999", b"-2147483648", b"1e39", b"nan", b"inf", b"//", b"/", b"f", b"v", b"vn",
          b"usemtl", b"{", b"}", b"[", b"]", b'"', b",", b":", b"\n", b"\x00", b"\xff", b"#", b"1/2/3",
          b"-5/-5/-5", b"0/0/0", b"-Y 100000 +X 100000", b"+Y 3 -X 2", b"\x02\x02", b"\x01\x01\x01\xff"]
for seed in range(seeds):
    rng = random.Random(seed)
    shutil.rmtree(work, ignore_errors=True)
    shutil.copytree(base, work)
    cfg = work / "s.json"
    cfg.write_text(cfg.read_text().replace(str(base), str(work)))
    target = work / rng.choice(names)
    b = bytearray(target.read_bytes())
    for _ in range(rng.randint(1, 6)):
        pos = rng.randrange(len(b) + 1)
        k = rng.random()
        if k < 0.25:
            b[pos:pos + 1] = bytes([rng.randrange(256)])
        elif k < 0.4:
            del b[pos:]
        elif k < 0.7:
            b[pos:pos] = rng.choice(tokens)
        elif k < 0.85:
            del b[pos:pos + rng.randint(1, 64)]
        else:
            b[pos:pos] = b[pos:pos + rng.randint(1, 256)] * rng.randint(1, 4)
    target.write_bytes(bytes(b))
    print("seed", seed, target.name, flush=True)
    try:
        Scene.load_json(cfg).arrays()
    except TTError:
        pass
"""


def test_mutated_inputs_load_or_fail_cleanly(tmp_path):
    """Seeded mutations (byte flips, truncation, inserted tokens, deleted and repeated spans) of a
    scene's JSON config, OBJ, material JSON and RGBE picture. Each load must succeed or raise
    TTError; it runs in a child process so that a crash fails this test instead of the run."""
    from tests.golden import rgbe_files

    base = tmp_path / "base"
    base.mkdir()
    cfg_path = _tricky_obj(base)
    hdr = rgbe_files.write_all(tmp_path)["mixed"]
    (base / "sky.hdr").write_bytes(hdr.read_bytes())
    cfg = json.loads(cfg_path.read_text())
    cfg["hdr-file-name"] = str(base / "sky.hdr")
    cfg["objects"].append({"type": "Sphere", "radius": 0.5, "position": [1.0, 0.5, 0.0], "material": "a"})
    cfg_path.write_text(json.dumps(cfg))
    Scene.load_json(cfg_path)  # the unmutated scene loads
    pr = subprocess.run([sys.executable, "-c", _MUTATE_AND_LOAD, str(base), str(tmp_path / "work"), "2000"],
                        capture_output=True, text=True, timeout=600, cwd=ROOT,
                        env={**os.environ, "PYTHONPATH": str(ROOT)})
    seen = [line for line in pr.stdout.splitlines() if line.startswith("seed")]
    assert pr.returncode == 0, (seen[-1:], pr.stderr[-2000:])
    assert len(seen) == 2000


def _random_obj_scene(rng, d: Path) -> Path:
    """A random OBJ in the forms the reference's loader reads (OBJLoader.cpp): several vertices on
    one `v` line, floats as repr / %f / %e / %E / %g with a sign / integers / "1." / ".5", tabs and
    runs of blanks, CRLF or LF, a last line with or without its end of line, ignored `vt` / `vp` /
    `s` / `o` / comment lines, faces of 3-6
    corners whose corners mix `v`, `v/t` and `v/t/n` (the texture and normal index of a corner
    without them carry over from the previous corner of the line), and material switches."""
    def num(x):
        k = int(rng.integers(8))
        if k == 0:
            return repr(float(np.float32(x)))
        if k == 1:
            return "%.6f" % x
        if k == 2:
            return "%e" % x
        if k == 3:
            return ("+" if x >= 0 else "") + "%.4g" % x
        if k == 4:
            return "%.3E" % x
        if k == 5:
            return str(int(round(x)))
        s = "%.5f" % x
        if k == 6:
            return s.rstrip("0")
        return s.replace("0.", ".", 1) if s.startswith("0.") else s.replace("-0.", "-.", 1) if s.startswith("-0.") else s

    def sep():
        return [" ", "  ", "\t", " \t "][int(rng.integers(4))]

    nv = int(rng.integers(3, 60))
    verts = rng.uniform(-5, 5, (nv, 3))
    norms = rng.uniform(-1, 1, (nv, 3))
    lines = ["# random", "mtllib m.mtl"]
    i = 0
    while i < nv:
        k = min(nv - i, [1, 1, 1, 2, 3][int(rng.integers(5))])
        lines.append("v" + sep() + sep().join(num(c) for p in verts[i:i + k] for c in p) + ["", " ", "\t"][int(rng.integers(3))])
        i += k
        if rng.random() < 0.1:
            lines.append(["", "# c", "vt 0.5 0.5", "vp 0.1", "s off", "o thing"][int(rng.integers(6))])
    lines += ["vn" + sep() + sep().join(num(c) for c in p) for p in norms]
    groups = int(rng.integers(1, 4))
    for gi in range(groups):
        lines += [f"g grp{gi}", "usemtl " + "abc"[int(rng.integers(3))]]
        for _ in range(int(rng.integers(1, 12))):
            corners = []
            for _ in range(int(rng.integers(3, 7))):
                v, t, n = int(rng.integers(1, nv + 1)), int(rng.integers(1, 5)), int(rng.integers(1, nv + 1))
                form = int(rng.integers(5))
                corners.append(str(v) if form == 0 else f"{v}/{t}" if form == 1 else f"{v}/{t}/{n}")
            lines.append("f" + sep() + sep().join(corners) + ["", " "][int(rng.integers(2))])
        if gi == groups - 1 and rng.random() < 0.3:
            lines.append("usemtl " + "abc"[int(rng.integers(3))])
    eol = "\r\n" if rng.random() < 0.5 else "\n"
    end = [eol, "", eol + eol + "   " + eol + "# end"][int(rng.integers(3))]  # the file's last line may lack one
    (d / "m.obj").write_bytes((eol.join(lines) + end).encode())
    (d / "m.mtl").write_text(json.dumps({"a": {"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]},
                                         "b": {"type": "Spec", "color": [0.9, 0.9, 0.9]},
                                         "c": {"type": "Diff", "diffuseColor": [0.2, 0.7, 0.2]}}))
    objects = []
    for _ in range(int(rng.integers(1, 4))):  # the same file placed up to three times
        tr = {}
        if rng.random() < 0.8:
            tr["scale"] = [float(x) for x in rng.uniform(0.2, 3, 3)]
        if rng.random() < 0.8:
            tr["orientation"] = [float(x) for x in rng.uniform(-180, 180, 3)]
        if rng.random() < 0.8:
            tr["translate"] = [float(x) for x in rng.uniform(-10, 10, 3)]
        objects.append({"type": "Mesh", "file": str(d / "m.obj"), **({"transform": tr} if tr else {})})
    cfg = {"work-dir": str(d), "samples": 1, "material-file": str(d / "m.mtl"), "hdr-file-name": "",
           "bvh-reload": True, "material-reload": True,
           "camera": {"width": 8, "height": 8, "position": [0.0, 0.0, 0.0], "yaw": 0.0, "pitch": 0.0,
                      "focal": 1.0, "aperture": 0.0},
           "objects": objects}
    (d / "s.json").write_text(json.dumps(cfg))
    return d / "s.json"


_REFERENCE_ARRAYS = r"""
import sys, numpy as np
from oracle import refhost
for cfg in sys.argv[1:]:
    np.savez(cfg + ".ref.npz", **refhost.scene_arrays(cfg))
"""


@pytest.mark.skipif(not refhost.available(), reason="the reference's loader is not built on this host")
def test_random_objs_match_reference_loader(tmp_path):
    """200 random OBJs (`_random_obj_scene`) give the reference loader's arrays bit for bit. The
    reference runs in a child process: it prints as it loads, and would end the run on a crash."""
    rng = np.random.default_rng(2026)
    cfgs = []
    for k in range(200):
        d = tmp_path / f"s{k}"
        d.mkdir()
        cfgs.append(_random_obj_scene(rng, d))
    pr = subprocess.run([sys.executable, "-c", _REFERENCE_ARRAYS, *map(str, cfgs)], capture_output=True, timeout=600,
                        cwd=ROOT, env={**os.environ, "PYTHONPATH": str(ROOT)})
    assert pr.returncode == 0, pr.stderr[-2000:]
    for cfg in cfgs:
        ref = np.load(str(cfg) + ".ref.npz")
        mine = Scene.load_json(cfg).arrays()
        for k in ["vertices", "normals", "vidx", "nidx", "mat"]:
            a, b = np.asarray(mine[k]), np.asarray(ref[k])
            assert a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32)), (cfg, k)


_REFERENCE_MATERIALS = r"""
import sys, numpy as np
from oracle import refhost
for cfg in sys.argv[1:]:
    m, g = refhost.scene_materials(cfg)
    np.savez(cfg + ".mat.npz", materials=m, geometries=g)
"""


def _random_material(rng) -> dict:
    def num(lo, hi):
        x = float(rng.uniform(lo, hi))
        k = int(rng.integers(3))
        return x if k == 0 else float("%.2e" % x) if k == 1 else int(round(x))

    kind = ["Diff", "Metal", "Spec", "Refr", "Coat"][int(rng.integers(5))]
    m = {"type": kind}
    if kind in ("Diff", "Coat"):
        m["diffuseColor"] = [num(0, 1) for _ in range(3)]
    if kind in ("Metal", "Spec"):
        m["color"] = [num(0, 1) for _ in range(3)]
    if kind == "Coat":
        m["specularColor"] = [num(0, 1) for _ in range(3)]
    if rng.random() < 0.3:
        m["emission"] = [num(0, 50) for _ in range(3)]
    return m


def _random_name(rng) -> str:
    chars = "abcXYZ019_-"
    return "".join(chars[int(i)] for i in rng.integers(0, len(chars), int(rng.integers(1, 6))))


@pytest.mark.skipif(not refhost.available(), reason="the reference's loader is not built on this host")
def test_random_materials_and_objects_match_reference_loader(tmp_path):
    """40 random scenes: a master material file and per-OBJ material files of random names (the
    reference keeps each pool in name order) and kinds, with or without emission, planes and
    spheres using master materials, and meshes. Materials (kind, emission, colours), analytic
    objects (kind, material index, radius, points) and triangle material indices all equal the
    reference loader's, bit for bit."""
    rng = np.random.default_rng(99)
    cfgs = []
    for k in range(40):
        d = tmp_path / f"m{k}"
        d.mkdir()
        master = {}
        while len(master) < int(rng.integers(1, 7)):
            master[_random_name(rng)] = _random_material(rng)
        (d / "master.mtl").write_text(json.dumps(master))
        names = list(master)
        objects = []
        for j in range(int(rng.integers(0, 3))):
            pool = {}
            while len(pool) < int(rng.integers(1, 4)):
                pool[_random_name(rng)] = _random_material(rng)
            (d / f"o{j}.mtl").write_text(json.dumps(pool))
            lines = [f"mtllib o{j}.mtl", "v 0 0 0", "v 1 0 0", "v 0 1 0", "v 1 1 0", "vn 0 0 1", "vn 0 0 1",
                     "vn 0 0 1", "vn 0 0 1"]
            for gi, name in enumerate(pool):
                lines += [f"g g{gi}", f"usemtl {name}", "f 1/1/1 2/1/2 3/1/3", "f 2/1/2 4/1/4 3/1/3"]
            (d / f"o{j}.obj").write_text("\n".join(lines) + "\n")
            objects.append({"type": "Mesh", "file": str(d / f"o{j}.obj")})
        for _ in range(int(rng.integers(0, 5))):
            mat = names[int(rng.integers(len(names)))]
            if rng.random() < 0.5:
                objects.append({"type": "Sphere", "radius": float(rng.uniform(0.1, 3)),
                                "position": [float(x) for x in rng.uniform(-5, 5, 3)], "material": mat})
            else:
                objects.append({"type": "Plane", "material": mat,
                                **{p: [float(x) for x in rng.uniform(-5, 5, 3)] for p in ("p0", "p1", "p2")}})
        if not any(o["type"] == "Mesh" for o in objects):  # every scene holds triangles
            (d / "t.mtl").write_text(json.dumps({"t": {"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}}))
            (d / "t.obj").write_text("mtllib t.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0 1\nvn 0 0 1\n"
                                     "g g\nusemtl t\nf 1/1/1 2/1/2 3/1/3\n")
            objects.insert(int(rng.integers(len(objects) + 1)), {"type": "Mesh", "file": str(d / "t.obj")})
        cfg = {"work-dir": str(d), "samples": 1, "material-file": str(d / "master.mtl"), "hdr-file-name": "",
               "bvh-reload": True, "material-reload": True,
               "camera": {"width": 8, "height": 8, "position": [0.0, 0.0, 0.0], "yaw": 0.0, "pitch": 0.0,
                          "focal": 1.0, "aperture": 0.0},
               "objects": objects}
        (d / "s.json").write_text(json.dumps(cfg))
        cfgs.append(d / "s.json")
    pr = subprocess.run([sys.executable, "-c", _REFERENCE_MATERIALS, *map(str, cfgs)], capture_output=True, timeout=600,
                        cwd=ROOT, env={**os.environ, "PYTHONPATH": str(ROOT)})
    assert pr.returncode == 0, pr.stderr[-2000:]
    for cfg in cfgs:
        ref = np.load(str(cfg) + ".mat.npz")
        sc = Scene.load_json(cfg)
        mats = np.array([[m.kind, *m.emission, *m.color, *m.color2] for m in sc.materials_raw()], np.float32)
        geoms = np.array([[g.kind, g.material, g.radius, 0.0, *g.p0, *g.p1, *g.p2] for g in sc.geometries_raw()],
                         np.float32).reshape(-1, 13)
        assert np.array_equal(mats.view(np.uint32), ref["materials"].view(np.uint32)), cfg
        assert np.array_equal(geoms.view(np.uint32), ref["geometries"].view(np.uint32)), cfg
        assert np.array_equal(sc.arrays()["mat"], refhost.scene_arrays(str(cfg))["mat"]), cfg
