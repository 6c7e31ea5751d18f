"""The native path tracer's samplers against their stated densities, independently of the
oracle's C restatement (oracle/tt_oracle_pt.c).

tt_native_sample_probe runs the renderer's own device sampling code on queries made here. The
directions it returns are binned and compared by a chi-square goodness-of-fit test with the bin
probabilities that the densities below give. Those densities are written here in numpy from the
published formulas, not from this project's code:
- Lambert: cos(theta) / pi.
- GGX conductor, visible-normal sampling (Heitz 2018, "Sampling the GGX Distribution of Visible
  Normals"): D(h) G1(wo) / (4 cos(theta_o)), with D and Smith's G1 of Walter et al. 2007.
- Dielectric: reflection with the exact Fresnel probability, else refraction by Snell's law.
- Environment map: texel probability proportional to luminance x sin(theta of the texel's row),
  mapped to solid angle by the equirectangular Jacobian.
- PCG32: the published output of the PCG reference implementation's demo for
  pcg32_srandom_r(42, 54), and O'Neill's pcg32_random_r restated in Python.
Every test uses fixed seeds. A chi-square p-value below 1e-4 fails.
"""
import math

import numpy as np
import pytest

from trenchanttracer_gb300 import BVHCompact, DeviceBVH, Renderer, Scene, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
stats = pytest.importorskip("scipy.stats")

ROUGHNESS = [0.3, 0.5, 0.8]
INCIDENCE_DEG = [0.0, 45.0, 75.0]
MATERIALS = ([{"name": "lambert", "type": "Diff", "diffuseColor": [0.8, 0.5, 0.2]}]
             + [{"name": f"ggx{r}", "type": "GGX", "F0": [0.9, 0.7, 0.5], "roughness": r} for r in ROUGHNESS]
             + [{"name": "glass", "type": "Dielectric", "ior": 1.5}])
GGX0, GLASS = 1, 1 + len(ROUGHNESS)


@pytest.fixture(scope="module")
def renderer():
    mesh = scenes.cornell(subdiv=1)
    mesh.mat[:] = 0
    mesh.materials = MATERIALS
    sc = Scene.from_mesh(mesh)
    sc.set_env(scenes.sky_env(2048, 1024, sun_radiance=5e4, sun_diameter_deg=0.5))
    return Renderer(DeviceBVH(BVHCompact.build(sc, 1e-5, 1, 8)), sc), sc


def _uniforms(rng, n, k=3):
    """Uniform numbers in [0, 1) with 24 random bits, as the renderer's uniform() makes them."""
    return (rng.integers(0, 1 << 24, (n, k)) * (1.0 / 16777216.0)).astype(np.float32)


def _bsdf_queries(material, n, wo, count, rng, entering=1):
    q = np.zeros(count, Renderer.SAMPLE_PROBE_DTYPE)
    q["material"] = material
    q["entering"] = entering
    q["n"] = n
    q["wo"] = wo
    q["u"] = _uniforms(rng, count)
    return q


def _chi2(counts, expected, min_expected=5.0):
    """Pearson chi-square with the bins expecting fewer than min_expected pooled into one."""
    counts = np.asarray(counts, np.float64).ravel()
    expected = np.asarray(expected, np.float64).ravel()
    small = expected < min_expected
    c = np.r_[counts[~small], counts[small].sum()]
    e = np.r_[expected[~small], expected[small].sum()]
    keep = e > 0
    c, e = c[keep], e[keep]
    stat = float(((c - e) ** 2 / e).sum())
    return stat, float(stats.chi2.sf(stat, max(1, c.size - 1)))


def _sphere_hist(wi, n_theta, n_phi):
    """Counts of unit directions over (theta, phi) bins about +z."""
    theta = np.arccos(np.clip(wi[:, 2].astype(np.float64), -1.0, 1.0))
    phi = np.arctan2(wi[:, 1].astype(np.float64), wi[:, 0].astype(np.float64))
    it = np.minimum((theta / math.pi * n_theta).astype(int), n_theta - 1)
    ip = np.minimum(((phi + math.pi) / (2 * math.pi) * n_phi).astype(int), n_phi - 1)
    return np.bincount(it * n_phi + ip, minlength=n_theta * n_phi).reshape(n_theta, n_phi)


def _bin_probabilities(pdf, n_theta, n_phi, sub=16):
    """Integral of pdf(directions (m, 3)) over each (theta, phi) bin: midpoint rule on a
    sub x sub grid per bin, d(omega) = sin(theta) d(theta) d(phi)."""
    out = np.zeros((n_theta, n_phi))
    dt, dp = math.pi / n_theta, 2 * math.pi / n_phi
    ft = (np.arange(sub) + 0.5) / sub
    for i in range(n_theta):
        th = (i + ft) * dt
        phs = ((np.arange(n_phi)[:, None] + ft[None, :]) * dp - math.pi).ravel()
        T, P = np.meshgrid(th, phs, indexing="ij")
        d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
        v = pdf(d).reshape(sub, n_phi, sub) * np.sin(T).reshape(sub, n_phi, sub)
        out[i] = v.sum(axis=(0, 2)) * (dt / sub) * (dp / sub)
    return out


# ---- densities from the published formulas ----------------------------------------------------
def ggx_d(alpha2, cos_h):
    c2 = cos_h * cos_h
    den = c2 * (alpha2 - 1.0) + 1.0
    return np.where(cos_h > 0, alpha2 / (math.pi * den * den), 0.0)


def smith_g1(alpha2, c):
    c = np.maximum(c, 1e-12)
    return 2.0 * c / (c + np.sqrt(alpha2 + (1.0 - alpha2) * c * c))


def ggx_vndf_pdf(roughness, wo):
    alpha = roughness * roughness
    a2 = alpha * alpha
    co = wo[2]

    def pdf(wi):
        h = wi + wo[None, :]
        ln = np.linalg.norm(h, axis=1)
        h = h / np.maximum(ln, 1e-300)[:, None]
        ok = (ln > 1e-12) & (h @ wo > 0)
        return np.where(ok, ggx_d(a2, h[:, 2]) * smith_g1(a2, co) / (4.0 * co), 0.0)

    return pdf


def fresnel_dielectric(cos_i, eta):
    """Unpolarised Fresnel reflectance; eta = n_incident / n_transmitted."""
    s2t = eta * eta * (1.0 - cos_i * cos_i)
    if s2t >= 1.0:
        return 1.0
    ct = math.sqrt(1.0 - s2t)
    rs = (eta * cos_i - ct) / (eta * cos_i + ct)
    rp = (cos_i - eta * ct) / (cos_i + eta * ct)
    return 0.5 * (rs * rs + rp * rp)


# ---- tests ----------------------------------------------------------------------------------------
def test_pcg32_matches_published_sequence(renderer):
    r, _ = renderer
    q = np.zeros(4, Renderer.SAMPLE_PROBE_DTYPE)
    q["pcg_state"] = [42, 0, 0xDEADBEEFCAFEF00D, 7]
    q["pcg_seq"] = [54, 0, 0x123456789ABCDEF, 1 << 62]
    out = r.sample_probe(Renderer.PROBE_PCG32, q)
    # the PCG reference implementation's demo prints these for pcg32_srandom_r(42, 54)
    published = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]
    assert [int(x) for x in out["pcg_out"][0, :6]] == published

    def pcg32_python(initstate, initseq, count):
        mask = (1 << 64) - 1
        inc = ((initseq << 1) | 1) & mask

        def step(s):
            out_ = ((((s >> 18) ^ s) >> 27) & 0xFFFFFFFF)
            rot = s >> 59
            return (s * 6364136223846793005 + inc) & mask, ((out_ >> rot) | (out_ << ((-rot) & 31))) & 0xFFFFFFFF

        s, _ = step(0)
        s = (s + initstate) & mask
        s, _ = step(s)
        vals = []
        for _ in range(count):
            s, v = step(s)
            vals.append(v)
        return vals

    for i in range(4):
        assert [int(x) for x in out["pcg_out"][i]] == pcg32_python(int(q["pcg_state"][i]), int(q["pcg_seq"][i]), 8)


def test_lambert_directions_follow_cosine_density(renderer):
    r, _ = renderer
    rng = np.random.default_rng(1)
    n = 1 << 20
    out = r.sample_probe(Renderer.PROBE_BSDF, _bsdf_queries(0, [0, 0, 1], [0.3, 0.2, 0.933], n, rng))
    wi = out["wi"]
    assert np.allclose(np.linalg.norm(wi, axis=1), 1.0, atol=2e-6)
    assert (wi[:, 2] > 0).all()
    counts = _sphere_hist(wi, 18, 24)
    expected = n * _bin_probabilities(lambda d: np.maximum(d[:, 2], 0.0) / math.pi, 18, 24)
    stat, p = _chi2(counts, expected)
    print(f"\nLambert: chi2 {stat:.1f}, p {p:.3g}")
    assert p > 1e-4
    cos_t = wi[:, 2].astype(np.float64)
    assert np.allclose(out["pdf"], cos_t / math.pi, rtol=1e-5, atol=1e-7)
    assert np.allclose(out["eval_pdf"], out["pdf"], rtol=1e-5, atol=1e-7)
    # any normal: the frame keeps the cosine distribution (cos^2 theta is uniform on [0, 1])
    nr = rng.normal(size=(n, 3))
    nr /= np.linalg.norm(nr, axis=1, keepdims=True)
    q = _bsdf_queries(0, [0, 0, 1], [0, 0, 1], n, rng)
    q["n"] = nr
    q["wo"] = nr
    out = r.sample_probe(Renderer.PROBE_BSDF, q)
    c = np.einsum("ij,ij->i", out["wi"].astype(np.float64), nr)
    assert (c > -1e-6).all()
    stat, p = _chi2(np.histogram(np.clip(c, 0, 1) ** 2, 50, (0, 1))[0], np.full(50, n / 50))
    assert p > 1e-4


@pytest.mark.parametrize("ri", range(len(ROUGHNESS)))
@pytest.mark.parametrize("inc", INCIDENCE_DEG)
def test_ggx_directions_follow_visible_normal_density(renderer, ri, inc):
    r, _ = renderer
    rough = ROUGHNESS[ri]
    rng = np.random.default_rng(100 + 10 * ri + int(inc))
    n = 1 << 20
    th = math.radians(inc)
    wo = np.array([math.sin(th), 0.0, math.cos(th)])
    out = r.sample_probe(Renderer.PROBE_BSDF, _bsdf_queries(GGX0 + ri, [0, 0, 1], wo.astype(np.float32), n, rng))
    wi = out["wi"].astype(np.float64)
    assert np.allclose(np.linalg.norm(wi, axis=1), 1.0, atol=1e-5)
    nt, nph = 36, 48
    counts = _sphere_hist(wi, nt, nph)
    prob = _bin_probabilities(ggx_vndf_pdf(rough, wo), nt, nph)
    assert abs(prob.sum() - 1.0) < 2e-3  # the density covers the whole sphere
    stat, p = _chi2(counts, n * prob)
    print(f"\nGGX roughness {rough}, incidence {inc} deg: chi2 {stat:.1f}, p {p:.3g}")
    assert p > 1e-4
    # the stated pdf of each sample above the horizon, and the evaluator's, match the formula
    up = (wi[:, 2] > 1e-3) & (out["pdf"] > 0)
    ref = ggx_vndf_pdf(rough, wo)(wi[up])
    assert np.median(np.abs(out["pdf"][up] / ref - 1.0)) < 1e-4
    assert np.quantile(np.abs(out["pdf"][up] / ref - 1.0), 0.999) < 1e-2
    assert np.quantile(np.abs(out["eval_pdf"][up] / out["pdf"][up] - 1.0), 0.999) < 1e-3


@pytest.mark.parametrize("inc", [0.0, 30.0, 60.0, 85.0])
@pytest.mark.parametrize("entering", [1, 0])
def test_dielectric_reflects_with_fresnel_probability_and_refracts_by_snell(renderer, inc, entering):
    r, _ = renderer
    rng = np.random.default_rng(200 + int(inc) + 7 * entering)
    n = 1 << 20
    th = math.radians(inc)
    wo = np.array([math.sin(th), 0.0, math.cos(th)], np.float32)
    out = r.sample_probe(Renderer.PROBE_BSDF, _bsdf_queries(GLASS, [0, 0, 1], wo, n, rng, entering=entering))
    wi = out["wi"].astype(np.float64)
    eta = 1.0 / 1.5 if entering else 1.5
    F = fresnel_dielectric(math.cos(th), eta)
    refl = wi[:, 2] > 0
    frac = refl.mean()
    sigma = math.sqrt(max(F * (1 - F), 1e-12) / n)
    print(f"\ndielectric entering={entering} {inc} deg: reflected {frac:.5f}, Fresnel {F:.5f}")
    assert abs(frac - F) <= 5 * sigma + 1e-6
    mirror = np.array([-wo[0], -wo[1], wo[2]], np.float64)
    assert np.allclose(wi[refl], mirror, atol=2e-6)
    if (~refl).any():
        t = wi[~refl]
        sin_t = np.sqrt(t[:, 0] ** 2 + t[:, 1] ** 2)
        assert np.allclose(sin_t, eta * math.sin(th), atol=3e-6)  # Snell
        assert np.allclose(t[:, 1], 0.0, atol=1e-6) and (t[:, 0] * wo[0] <= 1e-7).all()  # in the plane, across


def test_environment_sampling_follows_luminance_times_sin_theta(renderer):
    r, sc = renderer
    env = sc.env().astype(np.float64)
    h, w = env.shape[:2]
    lum = 0.2126 * env[..., 0] + 0.7152 * env[..., 1] + 0.0722 * env[..., 2]
    st = np.sin((np.arange(h) + 0.5) / h * math.pi)
    wt = np.maximum(lum * st[:, None], 0.0)
    p_texel = wt / wt.sum()
    rng = np.random.default_rng(3)
    n = 1 << 23
    q = np.zeros(n, Renderer.SAMPLE_PROBE_DTYPE)
    q["u"] = _uniforms(rng, n)
    out = r.sample_probe(Renderer.PROBE_ENV, q)
    assert (out["pdf"] > 0).all()
    d = out["wi"].astype(np.float64)
    u = (np.arctan2(d[:, 0], d[:, 2]) % (2 * math.pi)) / (2 * math.pi)
    v = np.arccos(np.clip(d[:, 1], -1, 1)) / math.pi
    x = np.minimum((u * w).astype(int), w - 1)
    y = np.minimum((v * h).astype(int), h - 1)
    # 32 x 32-texel blocks, except that each texel of the sun's 8 x 8 block is its own bin
    sun = np.unravel_index(np.argmax(p_texel), p_texel.shape)
    blk = (y // 32) * (w // 32) + x // 32
    sy, sx = sun[0] // 8 * 8, sun[1] // 8 * 8
    in_sun = (y >= sy) & (y < sy + 8) & (x >= sx) & (x < sx + 8)
    nb = (h // 32) * (w // 32)
    key = np.where(in_sun, nb + (y - sy) * 8 + (x - sx), blk)
    counts = np.bincount(key, minlength=nb + 64)
    yy, xx = np.mgrid[0:h, 0:w]
    in_sun_t = (yy >= sy) & (yy < sy + 8) & (xx >= sx) & (xx < sx + 8)
    key_t = np.where(in_sun_t, nb + (yy - sy) * 8 + (xx - sx), (yy // 32) * (w // 32) + xx // 32)
    expected = n * np.bincount(key_t.ravel(), weights=p_texel.ravel(), minlength=nb + 64)
    stat, p = _chi2(counts, expected)
    print(f"\nenvironment ({w} x {h}, sun {p_texel[in_sun_t].sum():.3f} of the power): chi2 {stat:.1f}, p {p:.3g}")
    assert p > 1e-4
    # the stated solid-angle pdf: p(texel) w h / (2 pi^2 sin(theta)) at the sample's own theta
    sin_theta = np.sqrt(np.maximum(0.0, 1.0 - d[:, 1] ** 2))
    with np.errstate(divide="ignore"):
        ref = p_texel[y, x] * w * h / (2 * math.pi ** 2 * sin_theta)
    big = p_texel[y, x] > 1e-7
    assert np.median(np.abs(out["pdf"][big] / ref[big] - 1.0)) < 3e-4  # float CDF entries: ~1e-4
    assert np.quantile(np.abs(out["pdf"][big] / ref[big] - 1.0), 0.999) < 1e-2
    # env_pdf (what light sampling's MIS weight uses for a BSDF-sampled direction) agrees
    assert np.quantile(np.abs(out["eval_pdf"] / out["pdf"] - 1.0), 0.999) < 1e-3


def test_environment_guide_tables_give_the_full_inverse_cdf(renderer):
    """The environment sampler searches each CDF only between the entries of a guide table (the
    answers at u = k / g); the texel it picks must be the full inverse-CDF search's answer (the
    smallest i with cdf[i + 1] > u) for uniform draws and for draws placed exactly on CDF entries,
    on guide grid points and one ulp either side of them."""
    r, sc = renderer
    h, w = sc.env().shape[:2]
    marg, cond = r.env_tables(w, h)
    rng = np.random.default_rng(7)
    u1 = [rng.random(1 << 20, dtype=np.float32)]
    u2 = [rng.random(1 << 20, dtype=np.float32)]
    edges = np.concatenate([marg[1:-1], np.arange(1, 1024, dtype=np.float32) / np.float32(1024)])
    for e in (edges, np.nextafter(edges, np.float32(0)), np.nextafter(edges, np.float32(1))):
        u1.append(e.astype(np.float32))
        u2.append(rng.random(e.size, dtype=np.float32))
    rows = rng.integers(0, h, 4096)  # draws on the conditional CDFs' own entries
    for k in range(4):
        cols = rng.integers(1, w, rows.size)
        v = cond[rows, cols]
        if k == 1:
            v = np.nextafter(v, np.float32(0))
        elif k == 2:
            v = np.nextafter(v, np.float32(1))
        elif k == 3:
            v = (cols // 4).astype(np.float32) / np.float32(512)
        mid = ((marg[rows] + marg[rows + 1]) * np.float32(0.5)).astype(np.float32)
        u1.append(mid)
        u2.append(v.astype(np.float32))
    u1 = np.concatenate(u1)
    u2 = np.concatenate(u2)
    keep = (u1 < 1) & (u2 < 1) & (u1 >= 0) & (u2 >= 0)
    u1, u2 = u1[keep], u2[keep]
    q = np.zeros(u1.size, Renderer.SAMPLE_PROBE_DTYPE)
    q["u"][:, 0] = u1
    q["u"][:, 1] = u2
    out = r.sample_probe(Renderer.PROBE_ENV, q)
    y = np.minimum(np.searchsorted(marg[1:], u1, side="right"), h - 1)
    x = np.empty_like(y)
    for yy in np.unique(y):
        sel = y == yy
        x[sel] = np.minimum(np.searchsorted(cond[yy, 1:], u2[sel], side="right"), w - 1)
    has_row = marg[y + 1] > marg[y]
    assert (out["texel"][~has_row] == -1).all()
    got = out["texel"][has_row]
    want = (y * w + x)[has_row]
    assert has_row.mean() > 0.99
    assert np.array_equal(got, want), f"{(got != want).sum()} of {got.size} texels differ from the full search"
