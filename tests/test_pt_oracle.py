"""The native path tracer's CPU restatement (oracle/tt_oracle_pt.c), checked on its own against
physics, with no GPU: the GPU tests then require the device renderer to match it bit for bit.

- white furnace: a closed-form scene whose every pixel has radiance 1 (a Lambert sphere of
  albedo 1, or a smooth dielectric, under a uniform unit environment);
- a sphere of albedo 0.5 under the same light is 0.5 (one bounce off a convex body escapes);
- a GGX conductor with F0 = 1 keeps no more than it receives;
- environment light sampling with MIS leaves the mean of a Lambert sphere under a sky with a sun
  where BSDF sampling alone puts it (unbiased), with less noise.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from trenchanttracer_gb300 import BVHCompact, Scene, _lib, make_camera_meta, render_params, scenes

CAM = dict(width=24, height=24, position=[0.0, 0.0, 3.0], view=[0.0, 0.0, -1.0], fov=(40.0, 40.0))


def _tan_half(deg: float) -> float:
    return float(np.float32(math.tan(deg * 0.5 * math.pi / 180.0)))


def _render(material: dict, env: np.ndarray, spp: int, max_depth: int, seed: int, flags: int = 0) -> np.ndarray:
    v, t, n = scenes.displaced_icosphere(3, 1.0, [0.0, 0.0, 0.0], 1, 0.0)
    mesh = scenes.Mesh(v, n, t, t.copy(), np.zeros(len(t), np.uint32), [material])
    sc = Scene.from_mesh(mesh)
    sc.set_env(env)
    bvh = BVHCompact.build(sc, 1e-5, 1, 8)
    mats, geos = sc.materials_raw(), sc.geometries_raw()
    cam = make_camera_meta(**CAM)
    params = render_params(spp=spp, max_depth=max_depth, rr_depth=4, seed=seed)
    params.flags |= flags
    acc = oracle.render_native(bvh.arrays(), (_lib.Material * len(mats))(*mats),
                               (_lib.Geometry * len(geos))(*geos), env, cam, params, _tan_half(CAM["fov"][0]),
                               _tan_half(CAM["fov"][1]))
    return acc.reshape(CAM["height"], CAM["width"], 3) / spp


UNIFORM = np.ones((16, 32, 3), np.float32)


@pytest.mark.parametrize("material", [{"type": "Diff", "diffuseColor": [1.0, 1.0, 1.0]},
                                      {"type": "Dielectric", "ior": 1.5}])
def test_white_furnace(material):
    img = _render(material, UNIFORM, spp=128, max_depth=64, seed=3)
    assert abs(img.mean() - 1.0) < 0.01, img.mean()


def test_half_albedo_sphere_is_half():
    img = _render({"type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}, UNIFORM, spp=128, max_depth=16, seed=4)
    centre = img[9:15, 9:15]  # sphere pixels only
    assert abs(centre.mean() - 0.5) < 0.01, centre.mean()


def test_ggx_conductor_keeps_no_more_than_it_receives():
    img = _render({"type": "GGX", "F0": [1.0, 1.0, 1.0], "roughness": 0.4}, UNIFORM, spp=64, max_depth=16, seed=5)
    centre = img[9:15, 9:15].mean()
    assert 0.85 < centre <= 1.02, centre


def test_environment_sampling_with_mis_is_unbiased_and_less_noisy():
    """A Lambert sphere under a sky with a sun of 12 degrees: environment light sampling with MIS
    and BSDF sampling alone give the same mean over the sphere's pixels (BSDF sampling alone has a
    heavy tail from the rare sun hits, so it takes 3 x 4096 samples per pixel for a standard error
    near 0.7 %), and MIS has a far smaller per-pixel noise, measured between two renders of
    different seeds (about 8x smaller)."""
    env = scenes.sky_env(64, 32, sun_radiance=60.0, sun_diameter_deg=12.0)
    m = {"type": "Diff", "diffuseColor": [0.8, 0.8, 0.8]}
    sphere = (slice(8, 16), slice(8, 16))
    mis = [_render(m, env, spp=2048, max_depth=2, seed=10 + k) for k in range(2)]
    bsdf = [_render(m, env, spp=4096, max_depth=2, seed=20 + k, flags=_lib.RENDER_NO_ENV_SAMPLING) for k in range(3)]
    a = np.mean([x[sphere].mean() for x in mis])
    b = np.mean([x[sphere].mean() for x in bsdf])
    assert abs(a - b) < 0.03 * b, (a, b)
    noise_mis = (mis[0] - mis[1])[sphere].std()
    noise_bsdf = (bsdf[0] - bsdf[1])[sphere].std() * math.sqrt(2)  # at 2048 spp, as the MIS renders
    assert noise_mis < 0.5 * noise_bsdf, (noise_mis, noise_bsdf)
