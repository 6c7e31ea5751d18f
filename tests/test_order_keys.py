"""The ray-ordering key (tt_ray_order_keys, the host twin of the key the ordered trace variants
sort by), against a numpy restatement of its definition: the origin cell of a grid over the
scene bounds whose bits go to the longest remaining cell side first, above the 8-bit cell of a
16 x 16 octahedral direction map. Every step is single-precision IEEE arithmetic without
products feeding sums, so the restatement is exact."""
import math

import numpy as np
import pytest

from trenchanttracer_gb300 import ray_order_keys

F = np.float32


def origin_bits(n: int) -> int:
    ob = 13
    while ob > 6 and (1 << (ob + 9)) > n:
        ob -= 2
    return max(ob, 6)


def grid(lo, hi, ob):
    lo = np.asarray(lo, F)
    hi = np.asarray(hi, F)
    side = []
    for k in range(3):
        e = float(hi[k]) - float(lo[k])
        side.append(e if (math.isfinite(e) and e > 0.0) else 0.0)
    bits, axis_of = [0, 0, 0], []
    for _ in range(ob):
        best = 0
        for k in (1, 2):
            if side[k] > side[best]:
                best = k
        axis_of.append(best)
        bits[best] += 1
        side[best] *= 0.5
    mask = [0, 0, 0]
    for b, k in enumerate(axis_of):
        mask[k] |= 1 << (ob - 1 - b)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):  # IEEE: x / 0 is inf, 0 / 0 NaN
        scale = [F(np.float64(1 << bits[k]) / (np.float64(hi[k]) - np.float64(lo[k]))) if bits[k] else F(0)
                 for k in range(3)]
    qmax = [F((1 << bits[k]) - 1) for k in range(3)]
    return lo, scale, qmax, mask, bits


def deposit(q: np.ndarray, mask: int) -> np.ndarray:
    out = np.zeros_like(q)
    j = 0
    for bit in range(32):
        if mask >> bit & 1:
            out |= ((q >> np.uint32(j)) & np.uint32(1)) << np.uint32(bit)
            j += 1
    return out


def cell(x: np.ndarray, top) -> np.ndarray:
    # (unsigned)fminf(fmaxf(x, 0), top): fmaxf / fminf return the non-NaN operand
    return np.fmin(np.fmax(x, F(0)), F(top)).astype(np.uint32)


def keys_np(rays: np.ndarray, lo, hi) -> tuple[np.ndarray, int]:
    ob = origin_bits(rays.shape[0])
    glo, scale, qmax, mask, _ = grid(lo, hi, ob)
    r = rays.astype(F)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        dx, dy, dz = r[:, 3], r[:, 4], r[:, 5]
        s = (np.abs(dx) + np.abs(dy)) + np.abs(dz)
        ok = (s > F(0)) & (s < F(np.inf))
        u, v = dx / s, dz / s
        low = dy < F(0)
        fu = (F(1) - np.abs(v)) * np.where(u < F(0), F(-1), F(1))
        fv = (F(1) - np.abs(u)) * np.where(v < F(0), F(-1), F(1))
        u = np.where(low, fu, u)
        v = np.where(low, fv, v)
        qu = cell((u + F(1)) * F(8), 15)
        qv = cell((v + F(1)) * F(8), 15)
        dcell = np.where(ok, deposit(qu, 0xAA) | deposit(qv, 0x55), np.uint32(0))
        oc = np.zeros(rays.shape[0], np.uint32)
        for k in range(3):
            oc |= deposit(cell((r[:, k] - glo[k]) * scale[k], qmax[k]), mask[k])
    return (oc << np.uint32(8)) | dcell, 8 + ob


def random_rays(n: int, seed: int, spread: float = 3.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rays = np.zeros((n, 8), F)
    rays[:, 0:3] = rng.uniform(-spread, spread, (n, 3))
    rays[:, 3:6] = rng.standard_normal((n, 3))
    rays[:, 6] = 1e-4
    rays[:, 7] = 1e30
    return rays


def test_random_rays_match_the_restatement():
    rays = random_rays(20000, 3)
    got, bits = ray_order_keys(rays, [-2.0, -1.0, -2.5], [2.0, 1.5, 2.0])
    ref, ref_bits = keys_np(rays, [-2.0, -1.0, -2.5], [2.0, 1.5, 2.0])
    assert bits == ref_bits == 8 + 6
    assert np.array_equal(got, ref)
    assert got.max() < (1 << bits)
    # the rays spread over most origin and direction cells
    assert len(np.unique(got & 0xFF)) > 200 and len(np.unique(got >> 8)) > 50


def test_edge_directions_and_origins():
    d = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 1), (-1, -1, -1),
         (0.5, -0.5, 0), (np.nan, 1, 0), (np.inf, 0, 0), (1e-30, -1e-30, 1e-30), (3e38, 3e38, 0), (-0.0, -0.0, 1),
         (0.125, 0.75, -0.125), (-1, -2, 1)]
    o = [(0, 0, 0), (-2, -1, -2.5), (2, 1.5, 2), (np.nan, 0, 0), (1e30, -1e30, 0), (1.999999, 1.4999, 1.999),
         (-0.0, 0.0, -0.0)]
    rays = np.array([[*oo, *dd, 0.0, 1e30] for oo in o for dd in d], F)
    got, bits = ray_order_keys(rays, [-2.0, -1.0, -2.5], [2.0, 1.5, 2.0])
    ref, _ = keys_np(rays, [-2.0, -1.0, -2.5], [2.0, 1.5, 2.0])
    assert np.array_equal(got, ref)
    assert got.max() < (1 << bits)
    # zero, NaN and infinite directions go to direction cell 0; a NaN origin to origin cell 0
    with np.errstate(over="ignore", invalid="ignore"):
        s = np.abs(rays[:, 3:6]).sum(axis=1)
    bad = ~np.isfinite(s) | (s == 0)
    assert np.all(got[bad] & 0xFF == 0)
    assert np.all(got[np.isnan(rays[:, 0])] >> 8 == ref[np.isnan(rays[:, 0])] >> 8)


@pytest.mark.parametrize("lo,hi", [([0, 0, 0], [1, 0, 1]), ([0, 0, 0], [0, 0, 0]), ([0, np.nan, 0], [1, 1, 1]),
                                   ([-1e30, 0, 0], [1e30, 1, 1])])
def test_degenerate_bounds(lo, hi):
    rays = random_rays(3000, 5)
    got, _ = ray_order_keys(rays, lo, hi)
    ref, _ = keys_np(rays, lo, hi)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n,bits", [(1, 14), (1 << 16, 15), (1 << 18, 17), (1 << 20, 19), ((1 << 22) - 1, 19),
                                    (1 << 22, 21)])
def test_key_width_follows_the_ray_count(n, bits):
    rays = np.zeros((n, 8), F)
    rays[:, 4] = 1.0
    got, b = ray_order_keys(rays, [0, 0, 0], [1, 1, 1])
    assert b == bits == 8 + origin_bits(n)
    assert got.max() < (1 << b)


def test_terrain_box_gives_the_longest_sides_most_origin_bits():
    # the terrain ray-cast scene at world scale 8: 16 x 1.8 x 16 (x, y, z)
    lo, hi = [-8.0, 0.0, -8.0], [8.0, 1.8, 8.0]
    *_, bits = grid(lo, hi, origin_bits(1 << 22))
    assert bits == [6, 2, 5]
    rays = random_rays(50000, 9, spread=8.0)
    rays[:, 1] = np.abs(rays[:, 1]) * F(0.2)
    got, _ = ray_order_keys(rays, lo, hi)
    ref, _ = keys_np(rays, lo, hi)
    assert np.array_equal(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3000, 1 << 16, 1 << 22])
def test_device_keys_equal_host_keys(n):
    """The ordering kernels' key function on the GPU (tt_ray_order_keys_device) gives the host
    keys bit for bit, edge directions and origins included, for key widths 6 + 8 to 13 + 8."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from trenchanttracer_gb300 import _lib
    lo, hi = [-2.0, -1.0, -2.5], [2.0, 1.5, 2.0]
    d = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, -1, 0), (0, 0, -1), (-1, -1, -1), (np.nan, 1, 0), (np.inf, 0, 0),
         (1e-30, -1e-30, 1e-30), (3e38, 3e38, 0), (-0.0, -0.0, 1), (0.125, 0.75, -0.125)]
    o = [(0, 0, 0), (-2, -1, -2.5), (2, 1.5, 2), (np.nan, 0, 0), (1e30, -1e30, 0), (1.999999, 1.4999, 1.999)]
    edge = np.array([[*oo, *dd, 0.0, 1e30] for oo in o for dd in d], F)
    rays = random_rays(n, 11)
    rays[:edge.shape[0]] = edge
    host, bits = ray_order_keys(rays, lo, hi)
    dr = torch.from_numpy(rays).cuda()
    dk = torch.empty(n, dtype=torch.int32, device="cuda")
    lo_a, hi_a = np.array(lo, F), np.array(hi, F)
    dbits = C.c_int32()
    _lib.check(_lib.lib().tt_ray_order_keys_device(C.c_void_p(dr.data_ptr()), n, C.c_void_p(lo_a.ctypes.data),
                                                    C.c_void_p(hi_a.ctypes.data), C.c_void_p(dk.data_ptr()),
                                                    C.byref(dbits), None))
    torch.cuda.synchronize()
    assert dbits.value == bits
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), host)
