"""The reference-compatible path tracer against the reference's own pathTracingKernel.

Same scene, camera (CameraMeta), frame seed (RenderMeta: WangHash(frame), PI = 3.14156265f) and
starting accumulation buffer go to both kernels; with matched curand XORWOW streams the per-pixel
mean radiance must agree within 1e-4 relative (the bar for matched RNG streams).
"""
import numpy as np
import pytest

from oracle import refgpu
from trenchanttracer_gb300 import (BVHCompact, DeviceBVH, Renderer, Scene, camera_meta, make_camera_meta,
                                   render_meta, scenes)

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

needs_ref = pytest.mark.skipif(not refgpu.render_available(), reason="reference render cubin not built")


def _render_both(scene: Scene, cam, samples: int, frame: int = 1, leaf_max: int = 8):
    bvh = BVHCompact.build(scene, 1e-5, 1, leaf_max)
    dbvh = DeviceBVH(bvh)
    r = Renderer(dbvh, scene)
    meta = render_meta(frame, samples)
    npx = cam.width * cam.height
    init = np.zeros(3 * npx, np.float32)
    acc = torch.from_numpy(init.copy()).cuda()
    r.render_compat(cam, meta, acc)
    torch.cuda.synchronize()
    r.check()
    mine = acc.cpu().numpy()
    ref, _ = refgpu.render(bvh.arrays(), scene.materials_raw(), scene.geometries_raw(), scene.env(), cam, meta, init)
    return mine, ref


def _compare(mine, ref, w, h, what, max_beyond=1e-3, mean_rel=1e-4):
    covered = np.zeros((h, w), bool)
    covered[h - (h // 16) * 16:, :(w // 16) * 16] = True  # the reference renders whole 16x16 blocks only
    m = mine.reshape(h, w, 3)[covered]
    r = ref.reshape(h, w, 3)[covered]
    assert np.isfinite(m).all() and np.isfinite(r).all()
    rel = np.abs(m - r) / np.maximum(np.abs(r), 1e-6)
    bad = (rel > 1e-4).any(axis=1)
    exact = (m.view(np.uint32) == r.view(np.uint32)).all(axis=1)
    mean_m, mean_r = float(m.astype(np.float64).mean()), float(r.astype(np.float64).mean())
    print(f"\n{what}: {exact.mean():.5f} of pixels bit-identical, {bad.mean():.6f} beyond 1e-4 relative, "
          f"mean radiance {mean_m:.6f} vs {mean_r:.6f} (relative {abs(mean_m - mean_r) / max(abs(mean_r), 1e-6):.2e})")
    assert r.max() > 0
    assert bad.mean() <= max_beyond, f"{what}: {bad.sum()} of {bad.size} pixels differ by more than 1e-4 relative"
    assert abs(mean_m - mean_r) <= mean_rel * max(abs(mean_r), 1e-6) + 1e-6


@needs_ref
def test_cornell_box_matches_reference_kernel():
    mesh = scenes.cornell(subdiv=4)
    sc = Scene.from_mesh(mesh)
    cam = make_camera_meta(96, 80, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 38.0), aperture=0.0, focal=1.0)
    mine, ref = _render_both(sc, cam, samples=4)
    _compare(mine, ref, 96, 80, "cornell")


@needs_ref
def test_every_reference_material_with_env_dof_and_analytic_objects():
    mesh, geoms = scenes.material_showcase(subdiv=3)
    sc = Scene.from_mesh(mesh)
    # the reference knows Diff / Metal / Spec / Refr / Coat only: map the two additions to Diff
    mats = [dict(m) for m in mesh.materials]
    for m in mats:
        if m["type"] in ("GGX", "Dielectric"):
            m.update(type="Diff", diffuseColor=[0.5, 0.5, 0.5])
    sc.set_materials(mats)
    sc.set_geometries(geoms)
    sc.set_env(scenes.sky_env(128, 64, sun_radiance=40.0, sun_diameter_deg=6.0))
    cam = make_camera_meta(128, 64, [0.0, 1.0, 3.2], [0.0, -0.25, -1.0], fov=(55.0, 30.0), aperture=0.03,
                           focal=3.0)
    mine, ref = _render_both(sc, cam, samples=4, frame=3)
    _compare(mine, ref, 128, 64, "materials + env + depth of field")


@needs_ref
def test_json_scene_camera_matches_reference_kernel(golden_scene_files):
    sc = Scene.load_json(golden_scene_files["mixed"])
    sc.set_env(scenes.sky_env(64, 32, sun_radiance=20.0, sun_diameter_deg=12.0))  # the scene has no emitter
    cam = camera_meta(sc, 45.0)
    mine, ref = _render_both(sc, cam, samples=2, frame=7)
    _compare(mine, ref, cam.width, cam.height, "JSON scene (planes, sphere, transforms)")


def test_compat_render_is_deterministic():
    mesh = scenes.cornell(subdiv=3)
    sc = Scene.from_mesh(mesh)
    dbvh = DeviceBVH(BVHCompact.build(sc, 1e-5, 1, 8))
    r = Renderer(dbvh, sc)
    cam = make_camera_meta(64, 64, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 45.0))
    out = []
    for _ in range(2):
        acc = torch.zeros(64 * 64 * 3, dtype=torch.float32, device="cuda")
        r.render_compat(cam, render_meta(1, 2), acc)
        torch.cuda.synchronize()
        out.append(acc.cpu().numpy())
    assert np.array_equal(out[0], out[1])
    assert out[0].mean() > 0.01


@needs_ref
def test_render_speed_beside_reference_kernel():
    """The bench's Cornell view (512 x 512, 16 samples per frame): the reference's own
    pathTracingKernel, tt_render_compat (the same algorithm, bit-compatible) and the native
    wavefront tracer (its own algorithm: depth 8, roulette from 4, ordered queues), timed with CUDA
    events on the same GB300. Printed for the record; the assertion only guards against the port
    falling far behind the reference."""
    from trenchanttracer_gb300 import render_params
    sc = Scene.from_mesh(scenes.cornell(subdiv=5))
    bvh = BVHCompact.build(sc, 1e-5, 1, 8)
    r = Renderer(DeviceBVH(bvh), sc)
    cam = make_camera_meta(512, 512, [0.0, 0.0, 1.55], [0.0, 0.0, -1.0], fov=(45.0, 45.0))
    spp, npx = 16, 512 * 512
    init = np.zeros(3 * npx, np.float32)
    ref_ms = min(refgpu.render(bvh.arrays(), sc.materials_raw(), sc.geometries_raw(), sc.env(), cam,
                               render_meta(f, spp), init)[1] for f in (1, 2, 3))
    acc = torch.zeros(3 * npx, dtype=torch.float32, device="cuda")

    def timed(fn):
        best = 1e9
        for f in range(4):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn(f)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1)) if f else best
        r.check()
        return best

    compat_ms = timed(lambda f: r.render_compat(cam, render_meta(f + 1, spp), acc))
    old = r.launch
    r.set_launch(128, 16, 1 << 22, 1)
    native_ms = timed(lambda f: r.render_native(cam, render_params(spp=spp, sample_offset=f * spp, max_depth=8,
                                                                   rr_depth=4, seed=1), acc))
    r.set_launch(*old)
    rate = lambda ms: spp * npx / ms / 1e3
    print(f"\nCornell 512x512 x {spp} spp, Msamples/s: reference pathTracingKernel {rate(ref_ms):.1f} ({ref_ms:.2f} ms), "
          f"tt_render_compat {rate(compat_ms):.1f} ({compat_ms:.2f} ms), native {rate(native_ms):.1f} ({native_ms:.2f} ms)")
    assert compat_ms < 2.0 * ref_ms


@needs_ref
def test_multi_material_speed_and_parity_beside_reference_kernel():
    """The bench's multi-material view (8,192,002 triangles, 2048 x 1024 sky with sun, 1920 x
    1080) with its GGX and dielectric spheres given the reference's Metal and Refr kinds: the
    reference's own pathTracingKernel and tt_render_compat (its algorithm) on the same GB300, 4
    samples per pixel, parity within 1e-4 and the time of each printed."""
    import math
    mesh = scenes.multi_material(400, 5)
    mats = []
    for m in mesh.materials:
        if m["type"] == "GGX":
            mats.append({"name": m["name"], "type": "Metal", "color": m["F0"]})
        elif m["type"] == "Dielectric":
            mats.append({"name": m["name"], "type": "Refr"})
        else:
            mats.append(dict(m))
    sc = Scene.from_mesh(mesh)
    sc.set_materials(mats)
    sc.set_env(scenes.sky_env(2048, 1024, sun_radiance=5e4, sun_diameter_deg=0.5))
    w, h = 1920, 1080
    fy = 2.0 * math.degrees(math.atan(math.tan(math.radians(30.0)) * h / w))
    cam = make_camera_meta(w, h, [0.0, 14.0, 34.0], [0.0, -12.0, -34.0], fov=(60.0, fy))
    bvh = BVHCompact.build(sc, 1e-5, 1, 8)
    r = Renderer(DeviceBVH(bvh), sc)
    meta = render_meta(1, 4)
    init = np.zeros(3 * w * h, np.float32)
    ref, ref_ms = refgpu.render(bvh.arrays(), sc.materials_raw(), sc.geometries_raw(), sc.env(), cam, meta, init)
    ref_ms = min(ref_ms, refgpu.render(bvh.arrays(), sc.materials_raw(), sc.geometries_raw(), sc.env(), cam, meta,
                                       init)[1])
    acc = torch.from_numpy(init.copy()).cuda()
    r.render_compat(cam, meta, acc)  # warm
    best = 1e9
    for _ in range(2):
        acc = torch.from_numpy(init.copy()).cuda()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r.render_compat(cam, meta, acc)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    r.check()
    # 96 % of pixels come out bit-identical. The rest carry a 1-2 ulp difference in a refracted
    # direction (the two compilers contract the Refr arithmetic differently) that a later bounce
    # turns into a different path; seen through glass with a 5e4-radiance sun behind it, such a
    # path moves its pixel far, so up to 2 % of pixels may lie beyond 1e-4 while the image mean
    # still agrees within 1e-4.
    _compare(acc.cpu().numpy(), ref, w, h, "multi-material (reference kinds)", max_beyond=0.02)
    rate = lambda ms: 4 * w * h / ms / 1e3
    print(f"multi-material 1920x1080 x 4 spp, Msamples/s: reference pathTracingKernel {rate(ref_ms):.1f} "
          f"({ref_ms:.1f} ms), tt_render_compat {rate(best):.1f} ({best:.1f} ms)")
    assert best < ref_ms
