"""Traversal kernels on the GPU, through the C ABI, checked three ways:

1. the oracle's restatement in the reference kernel's arithmetic (small and medium cases);
2. tests/golden/trace_gpu_golden.npz, outputs of the reference's own kernel on a GB300;
3. the reference's own kernel run live (oracle/_ref/ref_intersect.cubin) at the full
   2,097,152-triangle terrain size, 4M coherent + 4M incoherent rays.
Hit ids and distances must be bit-identical; so must material indices and normals (ext).
"""
import ctypes as C
import json
import struct

import numpy as np
import pytest

from oracle import oracle, refgpu
from trenchanttracer_gb300 import BVHCompact, DeviceBVH, Scene, TTError, _lib, scenes

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def trace(dbvh, rays, closest, ext=False):
    d_rays = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    d_hits = torch.full((rays.shape[0], 6 if ext else 2), -7, dtype=torch.int32, device="cuda")
    dbvh.intersect(d_rays, d_hits, closest=closest, ext=ext)
    torch.cuda.synchronize()
    dbvh.check()
    h = d_hits.cpu().numpy()
    out = {"id": h[:, 0].copy()}
    if ext:
        out.update(mat=h[:, 1].copy(), t=h[:, 2].copy().view(np.float32), normal=h[:, 3:6].copy().view(np.float32))
    else:
        out["t"] = h[:, 1].copy().view(np.float32)
    return out


def assert_same(a, b, normals=False, what=""):
    assert np.array_equal(a["id"], b["id"]), f"{what}: {int((a['id'] != b['id']).sum())} id mismatches"
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32)), \
        f"{what}: {int((a['t'].view(np.uint32) != b['t'].view(np.uint32)).sum())} t mismatches"
    if normals:
        hit = a["id"] >= 0
        assert np.array_equal(a["mat"][hit], b["mat"][hit]), what
        assert np.array_equal(a["normal"].view(np.uint32)[hit], b["normal"].view(np.uint32)[hit]), what


class Case:
    def __init__(self, mesh, leaf_max=8):
        self.mesh = mesh
        self.bvh = BVHCompact.build(Scene.from_mesh(mesh), 1e-5, 1, leaf_max)
        self.arrays = self.bvh.arrays()
        self.dbvh = DeviceBVH(self.bvh)


@pytest.fixture(scope="module")
def cornell():
    return Case(scenes.cornell(5))


@pytest.fixture(scope="module")
def terrain_small():
    return Case(scenes.terrain(128, 8.0))


def small_ray_sets(case, kind):
    if kind == "cornell":
        prim = scenes.pinhole_rays(200, 150, [0.0, 0.0, 1.6], [0.0, 0.0, 0.0], 0.45)
        scale = 1.0
    else:
        scale = 8.0
        cam = scenes.terrain_camera(scale)
        prim = scenes.pinhole_rays(300, 301, cam["eye"], cam["target"], cam["tan_half_fov"])
    first = oracle.intersect(case.arrays, prim, True, normals=True)
    sec, _ = scenes.secondary_rays(prim, first["t"], first["normal"], prim.shape[0], 3, 1e-4 * scale)
    sets = {"primary": prim, "diffuse": sec,
            "shadow": scenes.shadow_rays(prim, first["t"], [0.1 * scale, 3.0 * scale, 0.2 * scale], 30011, 5,
                                         1e-4 * scale),
            "random": scenes.random_rays(40000, 9, [-1.3 * scale] * 3, [1.3 * scale] * 3)}
    return sets


@pytest.mark.parametrize("kind", ["cornell", "terrain"])
@pytest.mark.parametrize("closest", [True, False])
def test_kernel_matches_oracle(kind, closest, cornell, terrain_small):
    case = cornell if kind == "cornell" else terrain_small
    for name, rays in small_ray_sets(case, kind).items():
        mine = trace(case.dbvh, rays, closest, ext=True)
        ref = oracle.intersect(case.arrays, rays, closest, arith=oracle.DEVICE, normals=True)
        assert_same(mine, ref, normals=True, what=f"{kind}/{name}")
        plain = trace(case.dbvh, rays, closest, ext=False)
        assert_same(plain, ref, what=f"{kind}/{name} (id,t)")


def test_kernel_matches_reference_kernel_golden(golden_dir):
    path = golden_dir / "trace_gpu_golden.npz"
    if not path.exists():
        pytest.skip("trace_gpu_golden.npz not generated yet")
    g = np.load(path)
    cases = {}
    for name in sorted({k.split("__")[0] for k in g.files}):
        spec = (g[f"{name}__builder"].item(), g[f"{name}__args"].item())
        if spec not in cases:
            cases[spec] = Case(getattr(scenes, spec[0])(*json.loads(spec[1])))
        for closest in (True, False):
            key = f"{name}__{'closest' if closest else 'any'}"
            ref = {k: g[f"{key}_{k}"] for k in ["id", "t", "mat", "normal"]}
            assert_same(trace(cases[spec].dbvh, g[f"{name}__rays"], closest, ext=True), ref, normals=True, what=key)


@pytest.fixture(scope="module")
def terrain_full():
    case = Case(scenes.terrain(1024, 8.0))
    cam = scenes.terrain_camera(8.0)
    prim = scenes.pinhole_rays(2048, 2048, cam["eye"], cam["target"], cam["tan_half_fov"])
    first = trace(case.dbvh, prim, True, ext=True)
    sec, _ = scenes.secondary_rays(prim, first["t"], first["normal"], prim.shape[0], 11, 8e-4)
    # shadow rays from first hits to the point (8, 2, 0) of the unit terrain (x 8), tmax = the
    # distance: about 23 % of them are occluded
    shadow = scenes.shadow_rays(prim, first["t"], [64.0, 16.0, 0.0], prim.shape[0], 5, 8e-4)
    case.sets = {"primary": prim, "incoherent": sec, "shadow": shadow}
    return case


def _differ(a, b):
    return (a["id"] != b["id"]) | (a["t"].view(np.uint32) != b["t"].view(np.uint32))


@pytest.mark.skipif(not refgpu.available(), reason="reference cubin / loader not built")
@pytest.mark.parametrize("closest", [True, False])
def test_full_size_terrain_bit_identical_to_reference_kernel(terrain_full, closest):
    """4M coherent + 4M incoherent rays on the 2,097,152-triangle terrain.

    Our kernel equals the reference's per-ray algorithm (the oracle) on every ray. The
    reference kernel's own warp vote lets a lane keep visiting nodes with a stale hit distance,
    so on a few rays per ten million its result departs from its per-ray algorithm (a leaf box
    whose entry rounds above a nearly equal hit distance: the neighbouring triangle of a shared
    edge, one ulp apart). Everywhere else our ids, distances, materials and normals are its bits.
    """
    case = terrain_full
    for name, rays in case.sets.items():
        ref = refgpu.intersect(case.arrays, rays, closest)
        ora = oracle.intersect(case.arrays, rays, closest, arith=oracle.DEVICE)
        mine = trace(case.dbvh, rays, closest, ext=True)
        assert_same(mine, ora, what=f"terrain1024/{name} vs oracle")
        ref_dev = _differ(ref, ora)
        assert ref_dev.mean() <= 1e-6, f"{name}: reference departs from its per-ray algorithm on {ref_dev.sum()} rays"
        keep = ~ref_dev
        sub = lambda d: {k: v[keep] for k, v in d.items() if isinstance(v, np.ndarray) and v.shape[0] == rays.shape[0]}
        assert_same(sub(mine), sub(ref), normals=True, what=f"terrain1024/{name} vs reference kernel")
        for i in np.nonzero(ref_dev)[0]:  # each departure is a one-ulp near tie
            assert abs(int(ref["t"].view(np.int32)[i]) - int(ora["t"].view(np.int32)[i])) <= 4
        assert 0.05 < (ref["id"] >= 0).mean() < 0.99


@pytest.mark.skipif(not refgpu.available(), reason="reference cubin / loader not built")
def test_warp_vote_variant_against_reference_kernel(terrain_full, capsys):
    """The warp-vote variant does what the reference kernel does (a lane with a postponed leaf
    keeps visiting nodes until the warp votes), so it is compared with the live reference kernel
    on the same 4M + 4M terrain rays. Where the reference agrees with its per-ray algorithm, the
    vote variant agrees with both; on the reference's few departures (near ties decided by which
    lanes are active at a vote) the count it reproduces is printed, as it depends on how each
    build's warps re-converge."""
    case = terrain_full
    for name, rays in case.sets.items():
        for closest in (True, False):
            ref = refgpu.intersect(case.arrays, rays, closest)
            ora = oracle.intersect(case.arrays, rays, closest, arith=oracle.DEVICE)
            vote = trace_with(case.dbvh, rays, closest, DeviceBVH.VARIANT_WARP_VOTE)
            ref_dev = _differ(ref, ora)
            vote_dev = _differ(vote, ora)
            vote_ref = _differ(vote, ref)
            with capsys.disabled():
                print(f"\n{name} closest={closest}: reference departs from the per-ray result on {ref_dev.sum()} "
                      f"rays, the vote variant on {vote_dev.sum()}, vote vs reference differ on {vote_ref.sum()} "
                      f"(of {rays.shape[0]})")
            assert vote_dev.mean() <= 1e-5 and vote_ref.mean() <= 1e-5
            assert not (vote_ref & ~ref_dev & ~vote_dev).any()  # off the near ties, one answer
            for i in np.nonzero(vote_dev)[0]:  # each departure is a near tie, as the reference's are
                assert abs(int(vote["t"].view(np.int32)[i]) - int(ora["t"].view(np.int32)[i])) <= 4


def test_variants_agree_bit_for_bit(terrain_full):
    """Every kernel variant except the warp-vote one yields the per-ray result."""
    case = terrain_full
    rays = case.sets["incoherent"][::4]
    ref = trace(case.dbvh, rays, True)
    default = case.dbvh.variant
    anyhit = trace(case.dbvh, rays, False)
    try:
        for v in DeviceBVH.DETERMINISTIC_VARIANTS:
            case.dbvh.set_variant(v)
            for closest in (True, False):
                assert_same(trace(case.dbvh, rays, closest), ref if closest else anyhit, what=f"variant {v}")
    finally:
        case.dbvh.set_variant(default)


def trace_with(dbvh, rays, closest, variant):
    old = dbvh.variant
    dbvh.set_variant(variant)
    try:
        return trace(dbvh, rays, closest)
    finally:
        dbvh.set_variant(old)


def test_full_size_properties(terrain_full):
    """Size-independent properties at the full size: any-hit finds a hit exactly when
    closest-hit does and never a nearer one; re-tracing is deterministic; clipping tmax to
    the closest distance removes the hit (the distance test is strict)."""
    case = terrain_full
    rays = case.sets["incoherent"]
    c1 = trace(case.dbvh, rays, True)
    c2 = trace(case.dbvh, rays, True)
    assert_same(c1, c2, what="determinism")
    a = trace(case.dbvh, rays, False)
    assert np.array_equal(c1["id"] >= 0, a["id"] >= 0)
    hit = c1["id"] >= 0
    assert (a["t"][hit] >= c1["t"][hit]).all()
    clipped = rays.copy()
    clipped[hit, 7] = c1["t"][hit]
    cc = trace(case.dbvh, clipped, True)
    assert (cc["t"][hit] <= c1["t"][hit]).all()
    assert (cc["id"][hit] == -1).mean() > 0.999


def test_host_path_full_size_matches_device_path(terrain_full):
    """The host-buffer entry point at 4M rays: coherent rays go in 1M-ray chunks in their own order,
    incoherent ones in growing chunks that are each ordered; every hit equals the device path's."""
    for name, rays in terrain_full.sets.items():
        dev = trace(terrain_full.dbvh, rays, True)
        hits = np.empty((rays.shape[0], 2), np.int32)
        terrain_full.dbvh.intersect_host(np.ascontiguousarray(rays), hits, closest=True)
        assert np.array_equal(hits[:, 0], dev["id"]), name
        assert np.array_equal(hits[:, 1], dev["t"].view(np.int32)), name
        # page-locked buffers: coherent rays are traced straight from and into host memory
        h_rays = torch.from_numpy(np.ascontiguousarray(rays)).pin_memory()
        h_hits = torch.full((rays.shape[0], 2), -7, dtype=torch.int32).pin_memory()
        terrain_full.dbvh.intersect_host(h_rays.numpy(), h_hits.numpy(), closest=True)
        assert np.array_equal(h_hits.numpy()[:, 0], dev["id"]), name + " (page-locked)"
        assert np.array_equal(h_hits.numpy()[:, 1], dev["t"].view(np.int32)), name + " (page-locked)"


def test_host_buffers_match_device_buffers(cornell):
    rays = small_ray_sets(cornell, "cornell")["diffuse"]
    hits = np.empty((rays.shape[0], 2), np.int32)
    cornell.dbvh.intersect_host(np.ascontiguousarray(rays), hits, closest=True)
    dev = trace(cornell.dbvh, rays, True)
    assert np.array_equal(hits[:, 0], dev["id"])
    assert np.array_equal(hits[:, 1], dev["t"].view(np.int32))


@pytest.mark.parametrize("n", [0, 1, 31, 33, 1000])
def test_ragged_batch_sizes(cornell, n):
    rays = scenes.random_rays(max(n, 1), 77, [-0.6] * 3, [0.6] * 3)[:n]
    if n == 0:
        d = torch.empty((0, 8), dtype=torch.float32, device="cuda")
        h = torch.empty((0, 2), dtype=torch.int32, device="cuda")
        cornell.dbvh.intersect(d, h)
        return
    assert_same(trace(cornell.dbvh, rays, True), oracle.intersect(cornell.arrays, rays, True), what=f"n={n}")


def test_edge_rays(cornell):
    """Axis-aligned directions (2^-80 guard), tmin > tmax (always a miss), origin on a wall,
    zero-length direction."""
    rays = scenes.random_rays(4096, 8, [-0.45] * 3, [0.45] * 3)
    rays[:1024, 3:6] = 0.0
    rays[np.arange(1024), 3 + np.arange(1024) % 3] = np.where(np.arange(1024) % 2, 1.0, -1.0)
    rays[1024:1536, 6] = 5.0
    rays[1024:1536, 7] = 1.0
    rays[1536:2048, 0:3] = [0.0, -0.5, 0.0]
    rays[2048:2100, 3:6] = 0.0
    for closest in (True, False):
        mine = trace(cornell.dbvh, rays, closest, ext=True)
        ref = oracle.intersect(cornell.arrays, rays, closest, normals=True)
        assert_same(mine, ref, normals=True, what="edge rays")
        # enough copies to go through the ray ordering (zero directions, rays out of the bounds)
        tiled = np.tile(rays, (10, 1))
        mine = trace(cornell.dbvh, tiled, closest, ext=True)
        ref_t = {k: np.concatenate([ref[k]] * 10) for k in ("id", "t", "mat", "normal")}
        assert_same(mine, ref_t, normals=True, what="edge rays, ordered")
        assert (mine["id"][1024:1536] == -1).all()


def test_empty_scene_and_unit_scale_cull():
    empty = BVHCompact.build(Scene.from_arrays(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3))), 1e-5, 1, 8)
    d = DeviceBVH(empty)
    r = scenes.random_rays(1000, 1, [-1] * 3, [1] * 3)
    assert (trace(d, r, True)["id"] == -1).all()
    # the reference accepts only det > 1e-5 (an absolute threshold): on a unit square a
    # 256^2-cell terrain has |e1 x e2| ~ 1.5e-5, so most triangles drop out at this scale
    case = Case(scenes.terrain(256, 0.5))
    cam = scenes.terrain_camera(0.5)
    prim = scenes.pinhole_rays(128, 128, cam["eye"], cam["target"], cam["tan_half_fov"])
    mine = trace(case.dbvh, prim, True)
    assert_same(mine, oracle.intersect(case.arrays, prim, True), what="unit scale")


def _self_loop_cache(path, child1_box_empty: bool):
    """A hand-made bvh.cache whose root lists itself as child 0 (and child 1): a corrupt file
    that passes the loader's address checks. The kernel's stack check / iteration cap must turn
    it into an error status instead of a hang or a fault. With `child1_box_empty` child 1's box
    lies far away from every test ray (an inverted box would not do: the slab test's min/max
    makes [hi, lo] the same box as [lo, hi]), so the ray loops on child 0 without pushing."""
    big = 1e3
    lo, hi = -big, big
    c1lo, c1hi = (1e6, 1e6 + 1.0) if child1_box_empty else (lo, hi)
    nodes = np.zeros((4, 4), np.float32)
    nodes[0] = [lo, hi, lo, hi]
    nodes[1] = [c1lo, c1hi, c1lo, c1hi]
    nodes[2] = [lo, hi, c1lo, c1hi]
    nodes_i = nodes.view(np.int32)
    nodes_i[3] = [0, 0, 0, 0]
    verts = np.array([[0x80000000, 0, 0, 0]], np.uint32).view(np.int32)
    with open(path, "wb") as f:
        f.write(struct.pack("<7I", 4, 0, 1, 1, 1, 1, 1))
        f.write(nodes_i.tobytes())
        f.write(verts.tobytes())
        f.write(verts.tobytes())
        f.write(np.zeros(1, np.int32).tobytes())
        f.write(np.zeros(1, np.uint32).tobytes())


@pytest.mark.parametrize("child1_empty,status", [(False, 5), (True, 4)])
def test_corrupt_bvh_reports_error_not_hang(tmp_path, child1_empty, status):
    p = tmp_path / "loop.cache"
    _self_loop_cache(p, child1_empty)
    d = DeviceBVH(BVHCompact.load(p))
    rays = scenes.random_rays(64, 3, [-1] * 3, [1] * 3)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((64, 2), dtype=torch.int32, device="cuda")
    d.intersect(d_rays, d_hits)
    with pytest.raises(TTError) as e:
        d.check()
    assert e.value.status == status  # 5 = TT_ERR_BOUNDS (stack), 4 = TT_ERR_TIMEOUT (iteration cap)
    assert (d_hits[:, 0] == -1).all()
    d.check()  # the error word was cleared; the context is still usable


@pytest.mark.skipif(not refgpu.available(), reason="reference cubin / loader not built")
def test_faster_than_reference_kernel(terrain_full, capsys):
    """Closest- and any-hit throughput of every terrain ray set against the reference's own
    kernel on the same GPU."""
    case = terrain_full
    out = {}
    for closest in (True, False):
        for name, rays in case.sets.items():
            ref = refgpu.intersect(case.arrays, rays, closest, reps=7)
            d_rays = torch.from_numpy(rays).cuda()
            d_hits = torch.empty((rays.shape[0], 2), dtype=torch.int32, device="cuda")
            ts = []
            for _ in range(7):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                case.dbvh.intersect(d_rays, d_hits, closest=closest)
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            mine = float(np.median(ts))
            out[(name, "closest" if closest else "any")] = (rays.shape[0] / mine / 1e3, rays.shape[0] / ref["ms"] / 1e3)
            assert mine < ref["ms"], f"{name} closest={closest}: {mine:.3f} ms vs reference {ref['ms']:.3f} ms"
    with capsys.disabled():
        print("\nMrays/s (ours, reference kernel):", {f"{k[0]}/{k[1]}": tuple(round(x) for x in v) for k, v in out.items()})
