"""The learned radiance cache on the GPU: its BF16 tensor-core kernels against the CPU oracle
(oracle/nrc_oracle.py), its training, and the path tracer that queries and trains it.

Tolerances: the device accumulates in FP32 in the tensor cores' order and rounds activations to
BF16 at the same points as the oracle (FP64), so a rounding boundary can fall differently for a
few values; the checks below bound the whole-vector error rather than demand equal bits.
"""
import numpy as np
import pytest

from oracle import nrc_oracle as nrc
from trenchanttracer_gb300 import BVHCompact, Cache, DeviceBVH, Renderer, Scene, make_camera_meta, render_params, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

LO, HI = [-2.0, -2.0, -2.0], [2.0, 2.0, 2.0]


def _records(n, seed):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 16), np.float32)
    rec[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    d = rng.normal(size=(n, 3))
    rec[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    m = rng.normal(size=(n, 3))
    rec[:, 6:9] = m / np.linalg.norm(m, axis=1, keepdims=True)
    rec[:, 9] = rng.uniform(0, 1, n)
    rec[:, 10:13] = rng.uniform(0, 1, (n, 3))
    rec[:, 13] = rng.integers(0, 7, n) / 8.0
    return rec


def _target(rec):
    ph = (rec[:, 0:3] + 2.0) / 4.0
    base = 0.6 + 0.5 * np.sin(2 * np.pi * ph[:, 0:1]) * np.cos(np.pi * ph[:, 2:3]) + 0.3 * rec[:, 4:5]
    return (np.exp(base) * rec[:, 10:13] + 0.05).astype(np.float32)


def _enc_np(cache, rec_t):
    return cache.encode(rec_t).float().cpu().numpy().astype(np.float64)


def test_encoding_matches_oracle():
    cache = Cache(LO, HI, batch=1024)
    rec = _records(1000, 1)
    got = _enc_np(cache, torch.from_numpy(rec).cuda())
    ref = nrc.bf16(nrc.encode(rec, LO, HI))
    diff = got != ref
    # FP32 sincospi versus FP64 sin/cos of the same argument: at most a neighbouring BF16 value
    assert diff.mean() < 1e-3, diff.mean()
    assert np.all(np.abs(got - ref)[diff] <= 2.0 ** -7 * np.abs(ref[diff]) + 1e-6)


def test_inference_matches_oracle():
    cache = Cache(LO, HI, batch=4096)
    w = nrc.init_weights(11)
    cache.set_weights(w)
    rec_t = torch.from_numpy(_records(3000, 2)).cuda()
    enc = _enc_np(cache, rec_t)
    got = cache.infer(rec_t).cpu().numpy()
    ref = nrc.radiance(enc, w)
    rel = np.abs(got - ref) / np.abs(ref)
    assert np.median(rel) < 1e-3 and rel.max() < 5e-2, (np.median(rel), rel.max())
    # the averaged weights equal the master weights right after set_weights
    assert torch.equal(cache.infer(rec_t, use_ema=True), cache.infer(rec_t))


@pytest.mark.parametrize("n", [1, 127, 128, 129, 3000])
def test_tcgen05_inference_matches_mma_sync_and_oracle(n):
    """The tcgen05 / TMEM inference kernel (mma_kind 0) against the mma.sync one (mma_kind 1) and
    the oracle, with the same BF16 weights, including partial 128-row tiles."""
    w = nrc.init_weights(21)
    tc = Cache(LO, HI, batch=4096, mma_kind=0)
    ms = Cache(LO, HI, batch=4096, mma_kind=1)
    tc.set_weights(w)
    ms.set_weights(w)
    rec_t = torch.from_numpy(_records(n, 7)).cuda()
    a = tc.infer(rec_t).cpu().numpy()
    b = ms.infer(rec_t).cpu().numpy()
    tc.check()
    ref = nrc.radiance(_enc_np(ms, rec_t), w)
    for got in (a, b):
        rel = np.abs(got - ref) / np.abs(ref)
        assert np.median(rel) < 1e-3 and rel.max() < 5e-2, (np.median(rel), rel.max())
    assert np.median(np.abs(a - b) / np.abs(b)) < 1e-3


def test_a_tensor_core_wait_that_runs_out_is_reported_and_the_context_stays_usable():
    """With a one-cycle budget every wait of the tcgen05 inference kernel runs out at once: the
    launch ends after its copies in flight have landed, tt_cache_check reports TT_ERR_TIMEOUT (once:
    the word is cleared), and on the same context a cache with the normal budget then agrees with
    the mma.sync kernel."""
    from trenchanttracer_gb300 import TTError
    w = nrc.init_weights(21)
    rec_t = torch.from_numpy(_records(3000, 7)).cuda()
    bad = Cache(LO, HI, batch=4096, mma_kind=0, wait_limit=1)
    bad.set_weights(w)
    bad.infer(rec_t)
    torch.cuda.synchronize()
    with pytest.raises(TTError, match="ran out"):
        bad.check()
    bad.check()  # reported once, then cleared
    tc = Cache(LO, HI, batch=4096, mma_kind=0)
    ms = Cache(LO, HI, batch=4096, mma_kind=1)
    tc.set_weights(w)
    ms.set_weights(w)
    a = tc.infer(rec_t).cpu().numpy()
    b = ms.infer(rec_t).cpu().numpy()
    tc.check()
    assert np.median(np.abs(a - b) / np.abs(b)) < 1e-3


def test_gradient_matches_oracle():
    cache = Cache(LO, HI, batch=4096)
    w = nrc.init_weights(12)
    cache.set_weights(w)
    rec = _records(2500, 3)
    tgt = _target(rec)
    rec_t, tgt_t = torch.from_numpy(rec).cuda(), torch.from_numpy(tgt).cuda()
    g, loss = cache.gradient(rec_t, tgt_t)
    assert np.array_equal(cache.weights(2), g)
    lref, gref = nrc.loss_and_gradient(_enc_np(cache, rec_t), w, tgt)
    assert abs(loss - lref) <= 1e-3 * lref
    off = nrc.offsets()
    for l in range(nrc.LAYERS):
        a, b = g[off[l]:off[l + 1]], gref[off[l]:off[l + 1]]
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < 2e-2, (l, err)
    assert not g[off[5] + 3 * 64:].any()  # padding rows of the output layer get no gradient


@pytest.mark.parametrize("n", [1, 129, 1000, 2500, 4096])
def test_tcgen05_training_matches_mma_sync_and_oracle(n):
    """The training pass on tcgen05 + TMEM (forward storing each layer's input, backward with the
    transposed weights, weight gradients with K = the batch's rows; mma_kind 0) against the
    mma.sync kernels (mma_kind 1) and the FP64 oracle, including partial 128-row tiles and
    1024-row gradient chunks; no wait runs out."""
    w = nrc.init_weights(31)
    tc = Cache(LO, HI, batch=4096, mma_kind=0)
    ms = Cache(LO, HI, batch=4096, mma_kind=1)
    tc.set_weights(w)
    ms.set_weights(w)
    rec = _records(n, 8)
    tgt = _target(rec)
    rec_t, tgt_t = torch.from_numpy(rec).cuda(), torch.from_numpy(tgt).cuda()
    g_tc, loss_tc = tc.gradient(rec_t, tgt_t)
    g_ms, loss_ms = ms.gradient(rec_t, tgt_t)
    tc.check()
    lref, gref = nrc.loss_and_gradient(_enc_np(ms, rec_t), w, tgt)
    assert abs(loss_tc - lref) <= 1e-3 * lref and abs(loss_tc - loss_ms) <= 1e-3 * loss_ms
    off = nrc.offsets()
    for l in range(nrc.LAYERS):
        a, b, r = g_tc[off[l]:off[l + 1]], g_ms[off[l]:off[l + 1]], gref[off[l]:off[l + 1]]
        assert np.linalg.norm(a - r) / np.linalg.norm(r) < 2e-2, (l, "vs oracle")
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-2, (l, "vs mma.sync")
    assert not g_tc[off[5] + 3 * 64:].any()  # padding rows of the output layer get no gradient


def test_adam_step_matches_oracle():
    cache = Cache(LO, HI, batch=2048, lr=1e-2, ema=0.5)
    w = nrc.init_weights(13)
    cache.set_weights(w)
    rec = _records(2048, 4)
    rec_t, tgt_t = torch.from_numpy(rec).cuda(), torch.from_numpy(_target(rec)).cuda()
    g, _ = cache.gradient(rec_t, tgt_t)
    cache.train(rec_t, tgt_t, steps=1)
    assert cache.steps == 1
    w1, _, _ = nrc.adam(w.astype(np.float64), 0.0, 0.0, g.astype(np.float64), 1, 1e-2)
    assert np.allclose(cache.weights(0), w1, rtol=1e-5, atol=1e-7)
    assert np.array_equal(cache.weights(1), cache.weights(0))  # the first average is the weights


def test_training_fits_a_radiance_field():
    cache = Cache(LO, HI, batch=4096, lr=5e-3)
    rec = _records(16384, 5)
    rec_t, tgt_t = torch.from_numpy(rec).cuda(), torch.from_numpy(_target(rec)).cuda()
    first = cache.train(rec_t, tgt_t, steps=4)
    for _ in range(60):
        last = cache.train(rec_t, tgt_t, steps=4)
    assert np.isfinite(last) and last < 0.1 * first, (first, last)
    test = _records(4096, 6)
    pred = cache.infer(torch.from_numpy(test).cuda(), use_ema=True).cpu().numpy()
    t = _target(test)
    assert np.mean((pred - t) ** 2 / (t * t + 0.01)) < 0.05


def _scene():
    mesh, geoms = scenes.material_showcase(subdiv=2)
    sc = Scene.from_mesh(mesh)
    sc.set_env(scenes.sky_env(64, 32, sun_radiance=60.0, sun_diameter_deg=12.0))
    bvh = BVHCompact.build(sc, 1e-5, 1, 8)
    r = Renderer(DeviceBVH(bvh), sc)
    lo, hi = mesh.vertices.min(0) - 0.1, mesh.vertices.max(0) + 0.1
    return r, lo, hi


CAM = dict(width=64, height=48, position=[0.0, 1.0, 3.2], view=[0.0, -0.25, -1.0], fov=(55.0, 42.0))


def test_cache_without_termination_is_the_plain_tracer():
    r, lo, hi = _scene()
    cache = Cache(lo, hi, spread_c=-1.0)
    cam = make_camera_meta(**CAM)
    p = render_params(spp=3, max_depth=6, rr_depth=3, seed=9)
    a = torch.zeros(64 * 48 * 3, dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    r.render_native(cam, p, a)
    r.render_cached(cache, cam, p, b, train=False)
    torch.cuda.synchronize()
    r.check()
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))


def _relmse(x, ref):
    return float(np.mean(np.sum((x - ref) ** 2 / (ref * ref + 1e-2), axis=-1)))


def test_trained_cache_beats_plain_tracing_at_equal_samples():
    """Paths end at their second vertex on the cache's estimate once it is trained: at equal
    samples per pixel the image is closer to a converged render than plain path tracing."""
    r, lo, hi = _scene()
    cam = make_camera_meta(**CAM)
    npx = 64 * 48 * 3
    ref = torch.zeros(npx, dtype=torch.float64, device="cuda")
    r.render_native(cam, render_params(spp=8192, max_depth=12, rr_depth=4, seed=1000, flags=1), ref)
    cache = Cache(lo, hi, train_paths=1024, batch=256, steps=4, spread_c=0.01)
    acc = torch.zeros(npx, dtype=torch.float32, device="cuda")
    for f in range(300):  # training frames
        acc.zero_()
        r.render_cached(cache, cam, render_params(spp=1, sample_offset=f, max_depth=12, rr_depth=4, seed=5), acc)
    torch.cuda.synchronize()
    r.check()
    assert cache.steps > 100
    spp = 16
    cached = torch.zeros(npx, dtype=torch.float32, device="cuda")
    for f in range(spp):
        r.render_cached(cache, cam, render_params(spp=1, sample_offset=300 + f, max_depth=12, rr_depth=4, seed=5),
                        cached)
    plain = torch.zeros(npx, dtype=torch.float32, device="cuda")
    r.render_native(cam, render_params(spp=spp, sample_offset=300, max_depth=12, rr_depth=4, seed=5), plain)
    torch.cuda.synchronize()
    ref_img = (ref.cpu().numpy() / 8192).reshape(-1, 3)
    e_cached = _relmse(cached.cpu().numpy().reshape(-1, 3) / spp, ref_img)
    e_plain = _relmse(plain.cpu().numpy().reshape(-1, 3) / spp, ref_img)
    assert np.isfinite(e_cached) and e_cached < e_plain, (e_cached, e_plain)


def test_cached_renders_with_training_are_reproducible():
    """Each training path owns a fixed record slot and the records reach the trainer in slot
    order, so two runs of trained, cached frames with fresh caches of the same seed give the same
    bits: images and weights (the queries' order does not matter: each path has at most one)."""
    r, lo, hi = _scene()
    cam = make_camera_meta(**CAM)
    npx = 64 * 48 * 3
    out = []
    for _ in range(2):
        cache = Cache(lo, hi, train_paths=1024, batch=256, steps=2, spread_c=0.01, seed=3)
        acc = torch.zeros(npx, dtype=torch.float32, device="cuda")
        for f in range(12):
            r.render_cached(cache, cam, render_params(spp=2, sample_offset=2 * f, max_depth=10, rr_depth=4, seed=7),
                            acc)
        torch.cuda.synchronize()
        r.check()
        cache.check()
        assert cache.steps > 0
        out.append((acc.cpu().numpy(), cache.weights(0), cache.weights(1)))
    (a0, w0, e0), (a1, w1, e1) = out
    assert a0.max() > 0
    assert np.array_equal(a0.view(np.uint32), a1.view(np.uint32))
    assert np.array_equal(w0.view(np.uint32), w1.view(np.uint32))
    assert np.array_equal(e0.view(np.uint32), e1.view(np.uint32))
