"""SBVH build and the compact layout: byte-identical bvh.cache against the reference builder.

The golden hashes in tests/golden/bvh_golden.json were written by the reference's own
SceneLoader + BVH + BVHCompact::save (tests/golden/make_golden.py). Where the reference's code is
built here (oracle/_ref), extra scenes are compared live.
"""
import hashlib
import json

import numpy as np
import pytest

from oracle import oracle, refhost
from tests.golden import golden_scenes
from trenchanttracer_gb300 import BVHCompact, Scene, TTError, scenes


def sha(p) -> str:
    return hashlib.sha256(open(p, "rb").read()).hexdigest()


@pytest.fixture(scope="module")
def golden(golden_dir):
    return json.loads((golden_dir / "bvh_golden.json").read_text())


@pytest.mark.parametrize("name", ["ico3", "terrain64", "cornell4", "mixed"])
@pytest.mark.parametrize("leaf_max", golden_scenes.LEAF_MAX)
def test_bvh_cache_matches_reference_builder(name, leaf_max, golden, golden_scene_files, tmp_path):
    sc = Scene.load_json(golden_scene_files[name])
    b = BVHCompact.build(sc, 1e-5, 1, leaf_max)
    out = tmp_path / "bvh.cache"
    b.save(out)
    ref = golden[name][str(leaf_max)]
    assert list(b.header.values()) == ref["header"]
    assert sha(out) == ref["sha256"]


@pytest.mark.parametrize("name", ["ico3", "terrain64", "cornell4", "mixed"])
@pytest.mark.parametrize("leaf_max", golden_scenes.LEAF_MAX)
def test_oracle_sbvh_matches_reference_builder(name, leaf_max, golden, golden_scene_files, tmp_path):
    """The oracle's own SBVH restatement (oracle/tt_oracle_sbvh.c, the host build bench.py's
    reference arm times) writes the reference builder's bvh.cache byte for byte."""
    a = Scene.load_json(golden_scene_files[name]).arrays()
    out = tmp_path / "oracle.cache"
    oracle.sbvh_build(a["vertices"], a["normals"], a["vidx"], a["nidx"], a["mat"], out, 1e-5, 1, leaf_max)
    ref = golden[name][str(leaf_max)]
    assert list(oracle.read_cache(out)["header"].values()) == ref["header"]
    assert sha(out) == ref["sha256"]


def test_oracle_sbvh_matches_product_builder_on_a_larger_terrain(tmp_path):
    """73,728 triangles: enough for the builder to split the root's axes over threads."""
    sc = Scene.from_mesh(scenes.terrain(192, 8.0, seed=11))
    a = sc.arrays()
    oracle.sbvh_build(a["vertices"], a["normals"], a["vidx"], a["nidx"], a["mat"], tmp_path / "o.cache", 1e-5, 1, 8)
    BVHCompact.build(sc, 1e-5, 1, 8).save(tmp_path / "p.cache")
    assert sha(tmp_path / "o.cache") == sha(tmp_path / "p.cache")


def test_signed_zero_and_tied_centroids_match_oracle(tmp_path):
    """Centroid sums of -0.0 and +0.0 compare equal in the reference's sort, so such references
    order by triangle index; the builder's radix sort of the root must agree. Half the triangles
    lie in the plane x = -0.0 or x = +0.0, a quarter are exact copies of others."""
    rng = np.random.default_rng(9)
    v = rng.uniform(-1, 1, (1800, 3)).astype(np.float32)
    v[:900:2, 0] = -0.0
    v[1:900:2, 0] = 0.0
    v[1350:] = v[:450]
    t = rng.permutation(1800).astype(np.int32).reshape(-1, 3)
    for leaf_min, leaf_max in [(1, 8), (1, 0x7FFFFFF), (3, 2)]:
        oracle.sbvh_build(v, v, t, t, np.zeros(600, np.uint32), tmp_path / "o.cache", 1e-5, leaf_min, leaf_max)
        BVHCompact.build(Scene.from_arrays(v, v, t), 1e-5, leaf_min, leaf_max).save(tmp_path / "p.cache")
        assert sha(tmp_path / "o.cache") == sha(tmp_path / "p.cache"), (leaf_min, leaf_max)


@pytest.mark.parametrize("name", ["ico3", "terrain64", "cornell4", "mixed"])
def test_scene_ingest_matches_reference_loader(name, golden, golden_scene_files):
    a = Scene.load_json(golden_scene_files[name]).arrays()
    digest = hashlib.sha256(b"".join(np.ascontiguousarray(a[k]).tobytes()
                                     for k in ["vertices", "normals", "vidx", "nidx", "mat"])).hexdigest()
    assert digest == golden[name]["scene_sha256"]


def test_build_is_independent_of_thread_count(tmp_path):
    sc = Scene.from_mesh(scenes.terrain(192, 8.0, seed=11))
    paths = []
    for threads in (1, 3, 0):
        p = tmp_path / f"t{threads}.cache"
        BVHCompact.build(sc, 1e-5, 1, 8, threads=threads).save(p)
        paths.append(sha(p))
    assert len(set(paths)) == 1


def test_cache_round_trip(tmp_path):
    sc = Scene.from_mesh(scenes.cornell(3))
    b = BVHCompact.build(sc, 1e-5, 1, 8)
    p = tmp_path / "a.cache"
    b.save(p)
    c = BVHCompact.load(p)
    assert c.header == b.header
    for k, v in b.arrays().items():
        assert np.array_equal(v, c.arrays()[k])
    # the independent reader used by the tests agrees
    raw = oracle.read_cache(p)
    assert raw["header"] == b.header


def test_layout_invariants():
    """Compact layout rules of BVHCompact::createCompact (src/bvh/BVHCompact.cpp:88-192)."""
    b = BVHCompact.build(Scene.from_mesh(scenes.terrain(32, 8.0)), 1e-5, 1, 8)
    a = b.arrays()
    hd = b.header
    nodes, verts = a["nodes"], a["vertices"]
    assert nodes.shape[0] % 4 == 0 and hd["nodes"] == nodes.shape[0]
    term = verts[:, 0].view(np.uint32) == 0x80000000
    assert term.sum() == hd["leaf_count"] and term[-1]
    assert (verts[term][:, 1:] == 0).all()
    assert hd["vertices"] == 3 * hd["tri_count"] + hd["leaf_count"]
    assert (verts[:, 3][~term] == 0).all()  # w = 0
    kids = nodes[3::4, :2].ravel()
    inner = kids[kids >= 0]
    assert (inner % 4 == 0).all() and inner.max() < nodes.shape[0]
    leaves = ~kids[kids < 0]
    assert leaves.max() < verts.shape[0]
    # every leaf address starts a run of whole triangles (3 slots each) ending at a terminator
    pos = np.nonzero(term)[0]
    next_term = pos[np.searchsorted(pos, leaves)]
    assert ((next_term - leaves) % 3 == 0).all()
    assert len(np.unique(leaves)) == hd["leaf_count"]
    assert (nodes[3::4, 2:] == 0).all()
    # tri indices: id, 0, 0 per triangle and 0 per terminator
    assert (a["tri_indices"][term] == 0).all()


def test_negative_zero_vertex_rewritten():
    """A -0.0 x coordinate of vertex 0 would read as the leaf terminator; the layout stores +0.0."""
    v = np.array([[-0.0, 0, 0], [1, 0, 0], [0, 0, 1], [-0.0, 1, 0]], np.float32)
    n = np.tile(np.array([[0, 1, 0]], np.float32), (4, 1))
    t = np.array([[0, 2, 1], [3, 0, 1]], np.int32)
    b = BVHCompact.build(Scene.from_arrays(v, n, t), 1e-5, 1, 8)
    a = b.arrays()
    xs = a["vertices"][:, 0].view(np.uint32)
    kids = a["nodes"][3::4, :2].ravel()
    # walk every leaf as the traversal does (slot 0 of each triangle is tested for the
    # terminator): the walk must cover every emitted triangle exactly once
    walked = 0
    for leaf in ~kids[kids < 0]:
        s = int(leaf)
        while xs[s] != 0x80000000:
            walked += 1
            s += 3
    assert walked == b.header["tri_count"] == 2
    # -0.0 survives in the other vertices (only vertex 0 is rewritten, BVHCompact.cpp:143)
    assert (xs == 0x80000000).sum() > b.header["leaf_count"]


@pytest.mark.parametrize("ntri", [0, 1, 2])
def test_tiny_scenes_get_an_inner_root(ntri):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1], [1, 0, 1]], np.float32)
    n = np.tile(np.array([[0, 1, 0]], np.float32), (4, 1))
    t = np.array([[0, 2, 1], [1, 2, 3]], np.int32)[:ntri]
    b = BVHCompact.build(Scene.from_arrays(v, n, t.reshape(-1, 3)), 1e-5, 1, 8)
    hd = b.header
    assert hd["nodes"] >= 4 and hd["tri_count"] == ntri


def test_rejects_bad_input(tmp_path):
    v = np.zeros((3, 3), np.float32)
    with pytest.raises(TTError):
        Scene.from_arrays(v, v, np.array([[0, 1, 5]], np.int32))
    # non-finite vertices are refused before any sort sees a NaN centroid
    rng = np.random.default_rng(1)
    for bad in (np.nan, np.inf, -np.inf):
        w = rng.uniform(-1, 1, (3000, 3)).astype(np.float32)
        w[1234, 1] = bad
        sc = Scene.from_arrays(w, w, np.arange(3000, dtype=np.int32).reshape(-1, 3))
        with pytest.raises(TTError) as e:
            BVHCompact.build(sc, 1e-5, 1, 8)
        assert e.value.status == 1 and "NaN or infinite" in str(e.value)
    p = tmp_path / "trunc.cache"
    good = tmp_path / "good.cache"
    BVHCompact.build(Scene.from_mesh(scenes.cornell(2)), 1e-5, 1, 8).save(good)
    raw = good.read_bytes()
    p.write_bytes(raw[:-5])
    with pytest.raises(TTError) as e:
        BVHCompact.load(p)
    assert e.value.status == 7
    bad = bytearray(raw)
    hdr = np.frombuffer(raw[:28], np.uint32)
    # corrupt the root's first child address to point past the node array
    off = 28 + 12 * 4
    bad[off:off + 4] = np.int32(4 * int(hdr[0]) + 8).tobytes()
    p.write_bytes(bytes(bad))
    with pytest.raises(TTError):
        BVHCompact.load(p)
    # a leaf address two entries before the end: in range, but its one "triangle" would read a
    # vertex past the array
    bad = bytearray(raw)
    bad[off:off + 4] = np.int32(~(int(hdr[3]) - 2)).tobytes()
    p.write_bytes(bytes(bad))
    with pytest.raises(TTError) as e:
        BVHCompact.load(p)
    assert "without a terminator" in str(e.value)
    # the last terminator overwritten: the walk from every leaf of the last run leaves the array
    bad = bytearray(raw)
    vstart = 28 + 16 * int(hdr[0])
    last = vstart + 16 * (int(hdr[3]) - 1)
    bad[last:last + 4] = np.float32(0.5).tobytes()
    p.write_bytes(bytes(bad))
    with pytest.raises(TTError):
        BVHCompact.load(p)


def _soup_scene(tmp_path, name, mesh):
    d = tmp_path / name
    d.mkdir()
    (d / "m.mtl").write_text(json.dumps(scenes.material_json(mesh.materials)))
    (d / "master.mtl").write_text(json.dumps({"w": {"type": "Diff", "diffuseColor": [1, 1, 1]}}))
    scenes.write_obj(str(d / "m.obj"), mesh, "m.mtl")
    cfg = {"work-dir": str(d), "samples": 1, "material-file": str(d / "master.mtl"), "hdr-file-name": "",
           "bvh-reload": True, "material-reload": True, "camera": {"width": 8, "height": 8},
           "objects": [{"type": "Mesh", "file": str(d / "m.obj"), "transform": {"scale": [5, 5, 5]}}]}
    (d / "s.json").write_text(json.dumps(cfg))
    return d / "s.json"


@pytest.mark.skipif(not refhost.available(), reason="the reference's builder is not built on this host")
@pytest.mark.parametrize("kind", ["soup", "flat", "dups", "copies"])
def test_live_against_reference_builder(kind, tmp_path):
    """Adversarial scenes: random triangle soup (spatial splits), a flat layer (zero-extent bins),
    duplicated triangles (ties in the sort key broken by triangle index) and 120 copies of one
    triangle, which with one triangle per leaf splits one off per level down to the depth limit.
    A leaf size floor above one makes leaves of the references in the order a node received them."""
    rng = np.random.default_rng(len(kind))
    if kind == "soup":
        v = rng.uniform(-1, 1, (900, 3)).astype(np.float32)
        t = np.arange(900, dtype=np.int32).reshape(-1, 3)
    elif kind == "flat":
        v = rng.uniform(-1, 1, (600, 3)).astype(np.float32)
        v[:, 1] = 0.25
        t = np.arange(600, dtype=np.int32).reshape(-1, 3)
    elif kind == "dups":
        base = rng.uniform(-1, 1, (150, 3)).astype(np.float32)
        v = np.concatenate([base, base, base])
        t = np.arange(450, dtype=np.int32).reshape(-1, 3)
    else:
        v = np.tile(rng.uniform(-1, 1, (3, 3)).astype(np.float32), (120, 1))
        t = np.arange(360, dtype=np.int32).reshape(-1, 3)
    mesh = scenes.Mesh(v, scenes._normalize(v + 3.0), t, t.copy(), np.zeros(len(t), np.uint32),
                       [{"name": "m", "type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}])
    cfg = _soup_scene(tmp_path, kind, mesh)
    for leaf_min, leaf_max in [(1, m) for m in golden_scenes.LEAF_MAX] + [(4, 1), (4, 8), (9, 16)]:
        refhost.build_json(str(cfg), str(tmp_path / "ref.cache"), 1e-5, leaf_min, leaf_max)
        BVHCompact.build(Scene.load_json(cfg), 1e-5, leaf_min, leaf_max).save(tmp_path / "new.cache")
        assert sha(tmp_path / "ref.cache") == sha(tmp_path / "new.cache"), (leaf_min, leaf_max)


@pytest.mark.skipif(not refhost.available(), reason="the reference's builder is not built on this host")
def test_random_scenes_and_settings_against_reference_builder(tmp_path):
    """Thirty random scenes (soups of small and large triangles, clustered and spread, some with
    duplicates) at random split alphas (0 lets every node try spatial splits; 1 almost none) and
    leaf settings: byte-identical bvh.cache files."""
    rng = np.random.default_rng(4242)
    for k in range(30):
        n = int(rng.integers(50, 1500))
        centres = rng.normal(0, 1, (n, 1, 3)) * (rng.uniform(0.2, 3, (1, 1, 3)) if k % 2 else 1.0)
        size = rng.uniform(0.01, 0.6) * (rng.lognormal(0, 1, (n, 1, 1)) if k % 3 == 0 else 1.0)
        v = (centres + rng.normal(0, 1, (n, 3, 3)) * size).reshape(-1, 3).astype(np.float32)
        if k % 4 == 1:
            v[-30:] = v[:30]  # ten repeated triangles
        t = np.arange(len(v), dtype=np.int32).reshape(-1, 3)
        mesh = scenes.Mesh(v, scenes._normalize(v + 3.0), t, t.copy(), np.zeros(len(t), np.uint32),
                           [{"name": "m", "type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}])
        cfg = _soup_scene(tmp_path, f"r{k}", mesh)
        alpha = float([0.0, 1e-7, 1e-5, 1e-3, 0.1, 1.0][int(rng.integers(6))])
        leaf_min = int(rng.integers(0, 6))
        leaf_max = int([1, 2, 4, 8, 16, 0x7FFFFFF][int(rng.integers(6))])
        refhost.build_json(str(cfg), str(tmp_path / "ref.cache"), alpha, leaf_min, leaf_max)
        BVHCompact.build(Scene.load_json(cfg), alpha, leaf_min, leaf_max).save(tmp_path / "new.cache")
        assert sha(tmp_path / "ref.cache") == sha(tmp_path / "new.cache"), (k, alpha, leaf_min, leaf_max)
