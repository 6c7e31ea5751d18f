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


def _compare(mine, ref, w, h, what):
    covered = np.zeros((h, w), bool)
    covered[h - (h // 16) * 16:, :(w // 16) * 16] = True  # the reference renders whole 16x16 blocks only
    m = mine.reshape(h, w, 3)[covered]
    r = ref.reshape(h, w, 3)[covered]
    assert np.isfinite(m).all() and np.isfinite(r).all()
    rel = np.abs(m - r) / np.maximum(np.abs(r), 1e-6)
    bad = (rel > 1e-4).any(axis=1)
    exact = (m.view(np.uint32) == r.view(np.uint32)).all(axis=1)
    print(f"\n{what}: {exact.mean():.5f} of pixels bit-identical, {bad.mean():.6f} beyond 1e-4 relative, "
          f"mean radiance {m.mean():.4f} vs {r.mean():.4f}")
    assert r.max() > 0
    assert bad.mean() <= 1e-3, f"{what}: {bad.sum()} of {bad.size} pixels differ by more than 1e-4 relative"
    assert abs(m.mean() - r.mean()) <= 1e-4 * max(abs(r.mean()), 1e-6) + 1e-6


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
