"""Pins the oracle before anything trusts it.

- Plain arithmetic against the reference's own intersect() compiled for the host
  (tests/golden/trace_host_golden.npz, written by tests/golden/make_golden.py).
- Device arithmetic (the FMA contraction nvcc applies on sm_103a) against the reference's own
  kernel run on a GB300 (tests/golden/trace_gpu_golden.npz, written by
  tests/golden/make_gpu_golden.py on the GPU host).
- WangHash values against the reference's WangHash::encode.
"""
import json

import numpy as np
import pytest

from oracle import oracle, refhost
from tests.golden import golden_scenes
from trenchanttracer_gb300 import BVHCompact, Scene

SCENES = ["ico3", "terrain64", "cornell4", "mixed"]


@pytest.fixture(scope="module")
def host_golden(golden_dir):
    return np.load(golden_dir / "trace_host_golden.npz")


@pytest.fixture(scope="module")
def bvhs(golden_scene_files):
    return {n: BVHCompact.build(Scene.load_json(golden_scene_files[n]), 1e-5, 1, golden_scenes.LEAF_MAX[-1]).arrays()
            for n in SCENES}


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("closest", [True, False])
def test_oracle_plain_matches_reference_host_intersect(name, closest, host_golden, bvhs):
    rays = host_golden[f"{name}_rays"]
    key = f"{name}_{'closest' if closest else 'any'}"
    o = oracle.intersect(bvhs[name], rays, closest, arith=oracle.PLAIN, normals=True)
    assert o["overflow"] == 0
    assert np.array_equal(o["id"], host_golden[f"{key}_id"])
    assert np.array_equal(o["t"].view(np.uint32), host_golden[f"{key}_t"].view(np.uint32))
    hit = o["id"] >= 0
    assert np.array_equal(o["mat"][hit], host_golden[f"{key}_mat"][hit])
    assert np.array_equal(o["normal"].view(np.uint32)[hit], host_golden[f"{key}_normal"].view(np.uint32)[hit])
    assert 0.02 < hit.mean() < 0.98  # the ray set exercises both hits and misses


def test_golden_rays_cover_edge_cases(host_golden):
    rays = host_golden["terrain64_rays"]
    assert (rays[:, 3:6] == 0).any()  # zero direction components (the 2^-80 guard)
    assert (rays[:, 6] > 0).any() and (rays[:, 6] == 0).any()


def test_wang_hash(golden_dir):
    cams = json.loads((golden_dir / "camera_golden.json").read_text())
    for a, v in cams["wang_hash"].items():
        assert oracle.wang_hash(int(a)) == v


def test_gpu_golden_pins_device_arithmetic(golden_dir):
    path = golden_dir / "trace_gpu_golden.npz"
    if not path.exists():
        pytest.skip("trace_gpu_golden.npz not generated yet")
    g = np.load(path)
    from trenchanttracer_gb300 import scenes
    built = {}
    for name in sorted({k.split("__")[0] for k in g.files}):
        spec = (g[f"{name}__builder"].item(), g[f"{name}__args"].item())
        if spec not in built:
            mesh = getattr(scenes, spec[0])(*json.loads(spec[1]))
            built[spec] = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, 8).arrays()
        arr = built[spec]
        for closest in (True, False):
            key = f"{name}__{'closest' if closest else 'any'}"
            rays = g[f"{name}__rays"]
            o = oracle.intersect(arr, rays, closest, arith=oracle.DEVICE, normals=True)
            assert np.array_equal(o["id"], g[f"{key}_id"]), key
            assert np.array_equal(o["t"].view(np.uint32), g[f"{key}_t"].view(np.uint32)), key
            hit = o["id"] >= 0
            assert np.array_equal(o["normal"].view(np.uint32)[hit], g[f"{key}_normal"].view(np.uint32)[hit]), key


@pytest.mark.skipif(not refhost.available(), reason="the reference's host code is not built on this host")
def test_live_oracle_against_reference_host(bvhs, golden_scene_files, tmp_path):
    """More rays than the fixture holds, straight against the reference's host-compiled code."""
    from trenchanttracer_gb300 import scenes
    name = "cornell4"
    b = BVHCompact.build(Scene.load_json(golden_scene_files[name]), 1e-5, 1, 8)
    b.save(tmp_path / "c.cache")
    rays = scenes.random_rays(60000, 99, [-1.2, -1.2, -1.2], [1.2, 1.2, 1.2])
    for closest in (True, False):
        r = refhost.intersect(str(tmp_path / "c.cache"), rays, closest)
        o = oracle.intersect(b.arrays(), rays, closest, arith=oracle.PLAIN)
        assert np.array_equal(r["id"], o["id"])
        assert np.array_equal(r["t"].view(np.uint32), o["t"].view(np.uint32))


def _edge_rays(count: int, seed: int, lo, hi) -> np.ndarray:
    """Random rays plus the cases the slab test treats specially: axis-aligned directions (zero
    components take the 2^-80 inverse-direction guard), negative zeros, directions of 1e-30,
    origins on box planes and at the scene's corners, t ranges that end before or start inside
    the scene, and an empty range (tmin = tmax)."""
    from trenchanttracer_gb300 import scenes
    rng = np.random.default_rng(seed)
    rays = scenes.random_rays(count, seed, lo, hi)
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    n = count // 8
    axes = np.eye(3, dtype=np.float32)[rng.integers(0, 3, n)] * rng.choice([-1.0, 1.0], (n, 1)).astype(np.float32)
    rays[:n, 3:6] = axes
    rays[n:2 * n, 3:6] = np.where(rng.random((n, 3)) < 0.5, np.float32(-0.0), rays[n:2 * n, 3:6])
    rays[2 * n:3 * n, 3:6] = np.where(rng.random((n, 3)) < 0.3, np.float32(1e-30), rays[2 * n:3 * n, 3:6])
    corner = np.where(rng.random((n, 3)) < 0.5, lo, hi)
    rays[3 * n:4 * n, 0:3] = corner
    rays[4 * n:5 * n, 6] = rng.uniform(0.0, 1.0, n).astype(np.float32)  # start inside the range
    rays[5 * n:6 * n, 7] = rng.uniform(0.0, 0.5, n).astype(np.float32)  # end early
    rays[6 * n:6 * n + 16, 6] = rays[6 * n:6 * n + 16, 7] = np.float32(0.25)
    return rays


@pytest.mark.skipif(not refhost.available(), reason="the reference's host code is not built on this host")
@pytest.mark.parametrize("kind", ["soup", "flat", "terrain"])
def test_live_oracle_on_edge_rays(kind, tmp_path):
    """The oracle against the reference's host-compiled intersect() on scenes with spatial splits,
    a flat layer (zero-extent boxes) and a terrain, with the slab test's special cases."""
    from trenchanttracer_gb300 import scenes
    rng = np.random.default_rng(len(kind))
    if kind == "terrain":
        mesh = scenes.terrain(48, 1.0, seed=5)
        v, t = mesh.vertices, mesh.vidx
    else:
        v = rng.uniform(-1, 1, (1500, 3)).astype(np.float32)
        if kind == "flat":
            v[:, 1] = 0.25
        t = np.arange(1500, dtype=np.int32).reshape(-1, 3)
    b = BVHCompact.build(Scene.from_arrays(v, v, t), 1e-5, 1, 8)
    b.save(tmp_path / "s.cache")
    lo, hi = v.min(0) - 0.1, v.max(0) + 0.1
    rays = _edge_rays(40000, 3 + len(kind), lo, hi)
    for closest in (True, False):
        r = refhost.intersect(str(tmp_path / "s.cache"), rays, closest)
        o = oracle.intersect(b.arrays(), rays, closest, arith=oracle.PLAIN, normals=True)
        assert np.array_equal(r["id"], o["id"]), (kind, closest)
        assert np.array_equal(r["t"].view(np.uint32), o["t"].view(np.uint32)), (kind, closest)
        hit = o["id"] >= 0
        assert hit.any() and (~hit).any()
        assert np.array_equal(r["normal"].view(np.uint32)[hit], o["normal"].view(np.uint32)[hit]), (kind, closest)
