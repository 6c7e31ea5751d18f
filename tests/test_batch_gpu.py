"""Batched rendering (tt_batch_*): many views of uneven size and sample count in one
graph-captured wavefront render.

Every view of a batch must be bit-identical to a plain tt_render_native of that view, whatever
the launch shape (block size, shared stack depth, paths per wave — including waves that split
pixels and views — ordered queues, waves or a streamed pool), with or without the CUDA graph;
the ray counters must agree too.
"""
import numpy as np
import pytest

from trenchanttracer_gb300 import Batch, BVHCompact, DeviceBVH, Renderer, Scene, make_camera_meta, render_params, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def showcase():
    mesh, geoms = scenes.material_showcase(subdiv=2)
    sc = Scene.from_mesh(mesh)
    sc.set_geometries(geoms)
    sc.set_env(scenes.sky_env(64, 32, sun_radiance=100.0, sun_diameter_deg=10.0))
    bvh = BVHCompact.build(sc, 1e-5, 1, 8)
    dbvh = DeviceBVH(bvh)
    return Renderer(dbvh, sc)


def _views(seed=0, count=7):
    rng = np.random.default_rng(seed)
    views = []
    for k in range(count):
        w, h = int(rng.integers(5, 40)), int(rng.integers(3, 30))
        yaw = float(rng.uniform(0, 2 * np.pi))
        pos = [3.0 * np.sin(yaw), float(rng.uniform(0.5, 2.0)), 3.0 * np.cos(yaw)]
        cam = make_camera_meta(w, h, pos, [-pos[0], 0.4 - pos[1], -pos[2]], fov=(50.0, 50.0 * h / w))
        views.append((cam, int(rng.choice([1, 2, 5])), int(rng.integers(0, 3)), int(rng.integers(1, 1000))))
    return views


PARAMS = dict(max_depth=5, rr_depth=2, env_scale=1.5)


def _sequential(r, views):
    imgs = []
    for cam, spp, off, seed in views:
        acc = torch.zeros(cam.width * cam.height * 3, dtype=torch.float32, device="cuda")
        r.render_native(cam, render_params(spp=spp, sample_offset=off, seed=seed, **PARAMS), acc)
        imgs.append(acc)
    torch.cuda.synchronize()
    r.check()
    return torch.cat(imgs).cpu().numpy()


def _batch(r, views, use_graph=True):
    b = Batch(r, views, render_params(**PARAMS))
    acc = torch.zeros(b.accum_elems, dtype=torch.float32, device="cuda")
    b.render(acc, use_graph=use_graph)
    torch.cuda.synchronize()
    r.check()
    return b, acc.cpu().numpy()


def test_batch_equals_sequential_renders(showcase):
    views = _views()
    seq = _sequential(showcase, views)
    b, got = _batch(showcase, views)
    assert b.total_paths == sum(c.width * c.height * s for c, s, _, _ in views)
    assert got.max() > 0 and np.isfinite(got).all()
    assert np.array_equal(got.view(np.uint32), seq.view(np.uint32))
    assert b.graph_kernels > 0
    _, plain = _batch(showcase, views, use_graph=False)
    assert np.array_equal(plain.view(np.uint32), seq.view(np.uint32))


@pytest.mark.parametrize("shape", [(64, 0, 777, 0, 0), (256, 8, 4096, 0, 1), (128, 16, 1 << 20, 0, 1),
                                   (64, 16, 31, 0, 0), (64, 16, 31, 0, 1), (64, 0, 777, 1, 1), (256, 8, 4096, 1, 0),
                                   (128, 16, 1 << 20, 1, 0), (64, 16, 31, 1, 1), (128, 16, 65536, 1, 1),
                                   (128, 16, 1000, 1, 1)])
def test_result_does_not_depend_on_launch_shape(showcase, shape):
    views = _views(seed=1, count=5)
    base = _sequential(showcase, views)
    old = showcase.launch
    try:
        showcase.set_launch(*shape)
        assert showcase.launch == shape
        _, got = _batch(showcase, views)
        seq = _sequential(showcase, views)
    finally:
        showcase.set_launch(*old)
    assert np.array_equal(got.view(np.uint32), base.view(np.uint32))
    assert np.array_equal(seq.view(np.uint32), base.view(np.uint32))


@pytest.mark.parametrize("wave,depth,ordered,f64", [(97, 5, 0, 0), (1000, 1, 0, 0), (4096, 12, 1, 0),
                                                    (50000, 5, 1, 0), (3001, 5, 0, 1), (65536, 9, 1, 1)])
def test_streamed_render_matches_waves(showcase, wave, depth, ordered, f64):
    """A render of more paths than one wave streams them through a pool of `wave` slots that is
    refilled as paths end (the queues mix paths of every age, and each path's radiance waits in
    a ring until all earlier paths have ended); the image must be bit-identical to the render in
    one wave, and the ray and path counters equal."""
    cam = make_camera_meta(64, 48, [2.0, 1.2, 2.5], [-2.0, -0.8, -2.5], fov=(50.0, 37.5))
    params = render_params(spp=7, sample_offset=3, seed=11, max_depth=depth, rr_depth=2, env_scale=1.5, flags=f64)
    dt = torch.float64 if f64 else torch.float32
    old = showcase.launch
    try:
        out = []
        for shape in [(128, 16, 1 << 22, 0), (64, 8, wave, ordered)]:
            showcase.set_launch(*shape)
            acc = torch.zeros(64 * 48 * 3, dtype=dt, device="cuda")
            showcase.stats(reset=True)
            showcase.render_native(cam, params, acc)
            torch.cuda.synchronize()
            showcase.check()
            out.append((acc.cpu().numpy(), showcase.stats(reset=True)))
    finally:
        showcase.set_launch(*old)
    (waves, s_waves), (streamed, s_streamed) = out
    assert waves.max() > 0
    assert np.array_equal(streamed.view(np.uint64 if f64 else np.uint32), waves.view(np.uint64 if f64 else np.uint32))
    assert s_streamed == s_waves and s_waves["paths"] == 64 * 48 * 7


def test_graph_replays_and_recaptures(showcase):
    views = _views(seed=2, count=4)
    b = Batch(showcase, views, render_params(**PARAMS))
    a1 = torch.zeros(b.accum_elems, dtype=torch.float32, device="cuda")
    a2 = torch.zeros_like(a1)
    b.render(a1)
    b.render(a2)  # new buffer: recaptured
    torch.cuda.synchronize()
    assert torch.equal(a1, a2)
    b.render(a1)  # replay into the first buffer again (a new graph for the old pointer)
    torch.cuda.synchronize()
    twice = a1.cpu().numpy()
    one = a2.cpu().numpy()
    assert np.allclose(twice, 2.0 * one, rtol=1e-5, atol=1e-6)


def test_f64_batch(showcase):
    views = _views(seed=3, count=3)
    b = Batch(showcase, views, render_params(flags=1, **PARAMS))
    acc = torch.zeros(b.accum_elems, dtype=torch.float64, device="cuda")
    b.render(acc)
    torch.cuda.synchronize()
    f32 = _sequential(showcase, views)
    assert np.allclose(acc.cpu().numpy(), f32, rtol=1e-5, atol=1e-6)


def test_ray_counters_and_autotune(showcase):
    views = _views(seed=4, count=6)
    showcase.stats(reset=True)
    seq = _sequential(showcase, views)
    s_seq = showcase.stats(reset=True)
    trials = Batch(showcase, views, render_params(**PARAMS)).autotune(sample_paths=20000)
    showcase.stats(reset=True)
    _, got = _batch(showcase, views)
    s_batch = showcase.stats(reset=True)
    assert s_seq == s_batch
    assert s_seq["paths"] == sum(c.width * c.height * s for c, s, _, _ in views)
    assert s_seq["extension_rays"] >= s_seq["paths"] and s_seq["shadow_rays"] > 0
    assert len(trials) >= 11 and all(t[5] > 0 for t in trials)
    assert {t[3] for t in trials} == {0, 1}
    stage1, stage2 = trials[:9], trials[9:]  # block x stack first, then waves / ordering / streaming
    assert {(t[0], t[1]) for t in stage1} == {(b, s) for b in (64, 128, 256) for s in (0, 8, 16)}
    assert {(t[0], t[1]) for t in stage2} == {min(stage1, key=lambda t: t[5])[:2]}
    best = min(stage2, key=lambda t: t[5])
    assert showcase.launch == best[:5]
    assert np.array_equal(got.view(np.uint32), seq.view(np.uint32))
