"""The native wavefront path tracer.

1. Bit-identical to the oracle's CPU restatement (oracle/tt_oracle_pt.c) on small images: same
   PCG32 streams, same float operations, same traversal, same accumulation order.
2. Physics checks the oracle cannot make by itself: white furnaces (Lambert albedo 1, a smooth
   dielectric: every path eventually escapes into a uniform unit environment, so the image is 1
   in expectation), an albedo-0.5 sphere (0.5), a GGX conductor with F0 = 1 (energy <= 1), and
   environment light sampling with MIS agreeing with BSDF sampling alone (unbiasedness).
"""
import math

import numpy as np
import pytest

from oracle import oracle
from trenchanttracer_gb300 import BVHCompact, DeviceBVH, Renderer, Scene, _lib, make_camera_meta, render_params, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _tan_half(deg: float) -> float:
    return float(np.float32(math.tan(deg * 0.5 * math.pi / 180.0)))


def _setup(scene: Scene):
    bvh = BVHCompact.build(scene, 1e-5, 1, 8)
    dbvh = DeviceBVH(bvh)
    return bvh, dbvh, Renderer(dbvh, scene)


def _render(r: Renderer, cam, params, f64=False):
    dtype = torch.float64 if f64 else torch.float32
    acc = torch.zeros(cam.width * cam.height * 3, dtype=dtype, device="cuda")
    r.render_native(cam, params, acc)
    torch.cuda.synchronize()
    r.check()
    return acc.cpu().numpy()


def _materials(scene: Scene):
    mats, geos = scene.materials_raw(), scene.geometries_raw()
    return (_lib.Material * len(mats))(*mats), (_lib.Geometry * len(geos))(*geos)


def _oracle(bvh, scene, env, cam, params):
    mats, geos = _materials(scene)
    return oracle.render_native(bvh.arrays(), mats, geos, env, cam, params, _tan_half(cam.fov[0]),
                                _tan_half(cam.fov[1]))


def test_native_matches_oracle_every_material_env_and_analytic_objects():
    mesh, geoms = scenes.material_showcase(subdiv=2)
    sc = Scene.from_mesh(mesh)
    sc.set_geometries(geoms)
    env = scenes.sky_env(64, 32, sun_radiance=200.0, sun_diameter_deg=8.0)
    sc.set_env(env)
    bvh, dbvh, r = _setup(sc)
    marg, cond = r.env_tables(64, 32)
    om, oc = oracle.env_tables(env)
    assert np.array_equal(marg.view(np.uint32), om.view(np.uint32))
    assert np.array_equal(cond.view(np.uint32), oc.view(np.uint32))
    cam = make_camera_meta(48, 32, [0.0, 1.0, 3.2], [0.0, -0.25, -1.0], fov=(55.0, 38.0))
    params = render_params(spp=4, max_depth=6, rr_depth=3, seed=11)
    gpu = _render(r, cam, params)
    cpu = _oracle(bvh, sc, env, cam, params)
    assert np.isfinite(gpu).all() and gpu.max() > 0
    diff = gpu.view(np.uint32) != cpu.view(np.uint32)
    assert not diff.any(), f"{diff.reshape(-1, 3).any(1).sum()} pixels differ from the oracle"


def test_native_matches_oracle_cornell_area_light():
    sc = Scene.from_mesh(scenes.cornell(subdiv=3))
    bvh, dbvh, r = _setup(sc)
    cam = make_camera_meta(40, 32, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 36.0))
    params = render_params(spp=8, max_depth=8, rr_depth=4, seed=3, sample_offset=5)
    gpu = _render(r, cam, params)
    cpu = _oracle(bvh, sc, None, cam, params)
    assert np.array_equal(gpu.view(np.uint32), cpu.view(np.uint32))
    assert gpu.mean() > 0


def test_native_thin_lens_matches_oracle():
    """The thin-lens camera (aperture > 1e-5) draws its lens sample after the pixel jitter; the
    device and the oracle must agree bit for bit, and the image must differ from the pinhole's."""
    sc = Scene.from_mesh(scenes.cornell(subdiv=3))
    bvh, dbvh, r = _setup(sc)
    cam = make_camera_meta(40, 32, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 36.0), aperture=0.06, focal=1.6)
    params = render_params(spp=6, max_depth=6, rr_depth=3, seed=21)
    gpu = _render(r, cam, params)
    cpu = _oracle(bvh, sc, None, cam, params)
    assert np.array_equal(gpu.view(np.uint32), cpu.view(np.uint32))
    pin = _render(r, make_camera_meta(40, 32, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 36.0)), params)
    assert not np.array_equal(pin, gpu)


def _sphere_scene(material: dict, radius=1.0) -> Scene:
    v, t, n = scenes.displaced_icosphere(4, radius, [0.0, 0.0, 0.0], 1, 0.0)
    mesh = scenes.Mesh(v, n, t, t.copy(), np.zeros(len(t), np.uint32), [material])
    sc = Scene.from_mesh(mesh)
    sc.set_env(np.ones((16, 32, 3), np.float32))
    return sc


FURNACE_CAM = dict(width=32, height=32, position=[0.0, 0.0, 3.0], view=[0.0, 0.0, -1.0], fov=(40.0, 40.0))


@pytest.mark.parametrize("material,expect", [
    ({"type": "Diff", "diffuseColor": [1.0, 1.0, 1.0]}, 1.0),
    ({"type": "Dielectric", "ior": 1.5}, 1.0),
])
def test_white_furnace(material, expect):
    sc = _sphere_scene(material)
    _, _, r = _setup(sc)
    cam = make_camera_meta(**FURNACE_CAM)
    spp = 256
    img = _render(r, cam, render_params(spp=spp, max_depth=64, rr_depth=4, seed=7)).reshape(32, 32, 3) / spp
    assert abs(img.mean() - expect) < 0.01, img.mean()


def test_half_albedo_sphere_is_half():
    sc = _sphere_scene({"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]})
    _, _, r = _setup(sc)
    cam = make_camera_meta(**FURNACE_CAM)
    spp = 256
    img = _render(r, cam, render_params(spp=spp, max_depth=16, rr_depth=4, seed=9)).reshape(32, 32, 3) / spp
    centre = img[12:20, 12:20]  # all sphere pixels
    assert abs(centre.mean() - 0.5) < 0.01, centre.mean()


def test_ggx_conductor_energy_bounded():
    sc = _sphere_scene({"type": "GGX", "F0": [1.0, 1.0, 1.0], "roughness": 0.4})
    _, _, r = _setup(sc)
    cam = make_camera_meta(**FURNACE_CAM)
    spp = 128
    img = _render(r, cam, render_params(spp=spp, max_depth=16, rr_depth=4, seed=5)).reshape(32, 32, 3) / spp
    centre = img[12:20, 12:20].mean()
    assert 0.85 < centre <= 1.02, centre


def test_env_light_sampling_is_unbiased():
    sc = _sphere_scene({"type": "Diff", "diffuseColor": [0.8, 0.8, 0.8]})
    sc.set_env(scenes.sky_env(128, 64, sun_radiance=500.0, sun_diameter_deg=6.0))
    _, _, r = _setup(sc)
    cam = make_camera_meta(**FURNACE_CAM)
    spp = 512
    a = _render(r, cam, render_params(spp=spp, max_depth=4, rr_depth=8, seed=1)) / spp
    b = _render(r, cam, render_params(spp=spp, max_depth=4, rr_depth=8, seed=2, flags=_lib.RENDER_NO_ENV_SAMPLING)) / spp
    assert abs(a.mean() - b.mean()) < 0.03 * b.mean(), (a.mean(), b.mean())
    assert a.std() < b.std()  # light sampling removes most of the sun's noise


def test_deterministic_and_f64_accumulation():
    mesh, geoms = scenes.material_showcase(subdiv=2)
    sc = Scene.from_mesh(mesh)
    sc.set_env(scenes.sky_env(64, 32))
    _, _, r = _setup(sc)
    cam = make_camera_meta(64, 48, [0.0, 1.0, 3.2], [0.0, -0.25, -1.0], fov=(55.0, 42.0))
    p = render_params(spp=3, seed=4)
    a, b = _render(r, cam, p), _render(r, cam, p)
    assert np.array_equal(a, b)
    d = _render(r, cam, render_params(spp=3, seed=4, flags=_lib.RENDER_ACCUM_F64), f64=True)
    assert np.allclose(d, a, rtol=1e-5, atol=1e-6)


def _many_analytic_objects(seed: int = 9) -> list:
    """About 90 analytic objects: random spheres of every material, tilted planes, a sphere listed
    twice (equal-t hits, where the lower index must win) and a plane lying on the ground mesh."""
    rng = np.random.default_rng(seed)
    geoms = []
    for _ in range(72):
        c = [float(rng.uniform(-3.5, 3.5)), float(rng.uniform(0.1, 2.5)), float(rng.uniform(-3.5, 1.0))]
        geoms.append({"type": "Sphere", "radius": float(rng.uniform(0.05, 0.3)), "position": c,
                      "material": int(rng.integers(1, 9))})
    geoms.append(dict(geoms[5]))
    geoms.insert(20, dict(geoms[30]))
    for _ in range(14):
        p0 = rng.uniform([-3.5, 0.0, -3.5], [3.5, 2.0, 0.5])
        e1, e2 = rng.normal(size=3) * 0.6, rng.normal(size=3) * 0.6
        geoms.append({"type": "Plane", "p0": [float(x) for x in p0], "p1": [float(x) for x in p0 + e1],
                      "p2": [float(x) for x in p0 + e2], "material": int(rng.integers(0, 8))})
    geoms.append({"type": "Plane", "p0": [-4.0, 0.0, -4.0], "p1": [4.0, 0.0, -4.0], "p2": [-4.0, 0.0, 4.0],
                  "material": 1})
    return geoms


def test_native_box_hierarchy_over_many_analytic_objects_matches_oracle():
    """More than 32 analytic objects go through the native tracer's box hierarchy instead of a
    loop over all of them per ray; the image must stay bit-identical to the oracle's loop."""
    mesh, _ = scenes.material_showcase(subdiv=2)
    sc = Scene.from_mesh(mesh)
    geoms = _many_analytic_objects()
    assert len(geoms) > 80
    sc.set_geometries(geoms)
    env = scenes.sky_env(64, 32, sun_radiance=200.0, sun_diameter_deg=8.0)
    sc.set_env(env)
    bvh, dbvh, r = _setup(sc)
    for cam in (make_camera_meta(48, 32, [0.0, 1.2, 3.4], [0.0, -0.2, -1.0], fov=(60.0, 42.0)),
                make_camera_meta(40, 40, [0.0, 6.0, 0.3], [0.0, -1.0, -0.05], fov=(70.0, 70.0))):
        params = render_params(spp=4, max_depth=6, rr_depth=3, seed=17)
        gpu = _render(r, cam, params)
        cpu = _oracle(bvh, sc, env, cam, params)
        assert np.isfinite(gpu).all() and gpu.max() > 0
        diff = gpu.view(np.uint32) != cpu.view(np.uint32)
        assert not diff.any(), f"{diff.reshape(-1, 3).any(1).sum()} pixels differ from the oracle"


def test_ordered_queues_give_the_same_image():
    """With ordered extension queues (every queue of 32K rays or more is ordered by direction and
    origin cell, traced, and its hits moved back) the image is bit-identical to the unordered
    render, and both to the oracle on a small crop of the same render."""
    sc = Scene.from_mesh(scenes.cornell(subdiv=4))
    bvh, dbvh, r = _setup(sc)
    cam = make_camera_meta(256, 256, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 45.0))
    params = render_params(spp=4, max_depth=6, rr_depth=3, seed=9)
    old = r.launch
    try:
        r.set_launch(128, 16, 1 << 22, 0)
        plain = _render(r, cam, params)
        r.set_launch(128, 16, 1 << 22, 1)
        assert r.launch[3] == 1
        ordered = _render(r, cam, params)
        r.set_launch(64, 0, 100000, 1, 0)  # waves that split the image, still above the ordering threshold
        ordered_waves = _render(r, cam, params)
        r.set_launch(64, 0, 100000, 1, 1)  # a streamed pool: the survivors ordered, new camera rays not
        ordered_streamed = _render(r, cam, params)
    finally:
        r.set_launch(*old)
    assert plain.max() > 0
    assert np.array_equal(ordered.view(np.uint32), plain.view(np.uint32))
    assert np.array_equal(ordered_waves.view(np.uint32), plain.view(np.uint32))
    assert np.array_equal(ordered_streamed.view(np.uint32), plain.view(np.uint32))
    small = make_camera_meta(24, 20, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 38.0))
    r.set_launch(128, 16, 1 << 22, 1)
    try:
        gpu = _render(r, small, params)
    finally:
        r.set_launch(*old)
    assert np.array_equal(gpu.view(np.uint32), _oracle(bvh, sc, None, small, params).view(np.uint32))


def test_launch_counter_matches_the_issued_sequence():
    """tt_renderer_launches counts the kernels a render issues: in waves, per wave raygen,
    accumulate and per bounce extend / shade / shadow (+ 4 ordering kernels and the hit gather, and
    with an environment 4 more for the shadow queue); streamed, an init, per iteration plan,
    accumulate, refill, extend, shade, shadow (+ the same ordering kernels) and a final plan and
    accumulate, over ceil(paths / pool) * depth + depth iterations."""
    import math
    sc = Scene.from_mesh(scenes.cornell(subdiv=2))
    sc.set_env(scenes.sky_env(32, 16))
    _, _, r = _setup(sc)
    cam = make_camera_meta(40, 30, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 35.0))
    depth, spp = 5, 3
    paths = 40 * 30 * spp
    params = render_params(spp=spp, max_depth=depth, rr_depth=3, seed=4)
    old = r.launch
    try:
        for wave, ordered, streamed in [(1 << 22, 0, 1), (1 << 22, 1, 1), (1000, 0, 0), (1000, 1, 0), (1000, 0, 1),
                                        (1000, 1, 1)]:
            r.set_launch(128, 16, wave, ordered, streamed)
            r.launches(reset=True)
            _render(r, cam, params)
            got = r.launches(reset=True)
            if streamed and paths > wave:
                iters = math.ceil(paths / wave) * depth + depth
                want = 1 + iters * (6 + (9 if ordered else 0)) + 2
            else:
                want = math.ceil(paths / wave) * (2 + depth * (12 if ordered else 3))
            assert got == want, (wave, ordered, streamed, got, want)
    finally:
        r.set_launch(*old)
