"""Seeded synthetic scenes and ray sets for the benchmark configurations.

Every generator uses only IEEE-exact float32 operations (+, -, *, /, sqrt, floor) and integer
hashing, never libm transcendentals, so the same seed yields the same bits on every host
(x86 development machines and Arm GPU hosts alike). Coordinates are world space, Y up, as in
the reference.

Scenes (the reference's assets are not available, so these stand in for them):
  terrain(n, scale)       n x n cell heightfield, 2 n^2 triangles, 6-octave fBm heights of
                          amplitude 0.1 over a unit square, seed 7; `scale` = world scale
                          (8 reproduces a unit-square OBJ normalised to [-1,1] and given a JSON
                          transform scale of 8, up to that loader's re-centring offset)
  icosphere(subdiv)       20 * 4^subdiv triangles on the unit sphere
  displaced_icosphere     icosphere with radial value-noise displacement
  cornell()               Cornell box walls + light + a displaced icosphere (config "small Cornell")
  multi_material()        400 displaced icospheres + ground, three material families
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

F = np.float32


# ---- hashing -------------------------------------------------------------------------------
def pcg_hash(x: np.ndarray) -> np.ndarray:
    """PCG-RXS-M-XS 32-bit hash (Jarzynski & Olano 2020), vectorised on uint32."""
    x = np.asarray(x, dtype=np.uint32)
    with np.errstate(over="ignore"):
        state = x * np.uint32(747796405) + np.uint32(2891336453)
        word = ((state >> ((state >> np.uint32(28)) + np.uint32(4))) ^ state) * np.uint32(277803737)
        return (word >> np.uint32(22)) ^ word


def hash_uniform(x: np.ndarray) -> np.ndarray:
    """uint32 -> float32 in [0, 1) with 24 random bits (exact)."""
    return (pcg_hash(x) >> np.uint32(8)).astype(F) * F(1.0 / 16777216.0)


def _lattice(ix: np.ndarray, iy: np.ndarray, iz: np.ndarray | None, seed: int) -> np.ndarray:
    h = pcg_hash(np.uint32(seed) + pcg_hash(ix.astype(np.uint32)))
    h = pcg_hash(h ^ iy.astype(np.uint32))
    if iz is not None:
        h = pcg_hash(h ^ iz.astype(np.uint32))
    return (h >> np.uint32(8)).astype(F) * F(2.0 / 16777216.0) - F(1.0)


def _smooth(t: np.ndarray) -> np.ndarray:
    return t * t * (F(3.0) - F(2.0) * t)


def value_noise2(x: np.ndarray, y: np.ndarray, seed: int) -> np.ndarray:
    """2D value noise in [-1, 1]: hashed lattice values, smoothstep-weighted bilinear blend."""
    x0 = np.floor(x)
    y0 = np.floor(y)
    fx = _smooth(x - x0)
    fy = _smooth(y - y0)
    ix = x0.astype(np.int64)
    iy = y0.astype(np.int64)
    v00 = _lattice(ix, iy, None, seed)
    v10 = _lattice(ix + 1, iy, None, seed)
    v01 = _lattice(ix, iy + 1, None, seed)
    v11 = _lattice(ix + 1, iy + 1, None, seed)
    a = v00 + (v10 - v00) * fx
    b = v01 + (v11 - v01) * fx
    return a + (b - a) * fy


def value_noise3(x, y, z, seed: int) -> np.ndarray:
    x0, y0, z0 = np.floor(x), np.floor(y), np.floor(z)
    fx, fy, fz = _smooth(x - x0), _smooth(y - y0), _smooth(z - z0)
    ix, iy, iz = x0.astype(np.int64), y0.astype(np.int64), z0.astype(np.int64)

    def lat(dx, dy, dz):
        return _lattice(ix + dx, iy + dy, iz + dz, seed)

    c00 = lat(0, 0, 0) + (lat(1, 0, 0) - lat(0, 0, 0)) * fx
    c10 = lat(0, 1, 0) + (lat(1, 1, 0) - lat(0, 1, 0)) * fx
    c01 = lat(0, 0, 1) + (lat(1, 0, 1) - lat(0, 0, 1)) * fx
    c11 = lat(0, 1, 1) + (lat(1, 1, 1) - lat(0, 1, 1)) * fx
    c0 = c00 + (c10 - c00) * fy
    c1 = c01 + (c11 - c01) * fy
    return c0 + (c1 - c0) * fz


def fbm2(x: np.ndarray, y: np.ndarray, octaves: int, seed: int) -> np.ndarray:
    """Fractal sum of `octaves` value-noise octaves (lacunarity 2, gain 0.5), in [-1, 1]."""
    total = np.zeros_like(x, dtype=F)
    amp = F(1.0)
    freq = F(1.0)
    norm = F(0.0)
    for o in range(octaves):
        total = total + amp * value_noise2(x * freq, y * freq, seed + 1013 * o)
        norm = norm + amp
        amp = amp * F(0.5)
        freq = freq * F(2.0)
    return total / norm


# ---- meshes ------------------------------------------------------------------------------
@dataclass
class Mesh:
    vertices: np.ndarray  # (V, 3) float32
    normals: np.ndarray   # (N, 3) float32
    vidx: np.ndarray      # (T, 3) int32
    nidx: np.ndarray      # (T, 3) int32
    mat: np.ndarray       # (T,) uint32
    materials: list = field(default_factory=list)  # list of dicts (material-JSON entries)

    @property
    def num_tris(self) -> int:
        return int(self.vidx.shape[0])


def _normalize(v: np.ndarray) -> np.ndarray:
    n = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    return (v / n[:, None]).astype(F)


def _cross(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1).astype(F)


def vertex_normals(vertices: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """Area-weighted smooth normals, accumulated in triangle order (deterministic)."""
    v0, v1, v2 = vertices[tris[:, 0]], vertices[tris[:, 1]], vertices[tris[:, 2]]
    fn = _cross(v1 - v0, v2 - v0)
    acc = np.zeros_like(vertices, dtype=F)
    for k in range(3):
        np.add.at(acc, tris[:, k], fn)
    return _normalize(acc)


def terrain(n: int = 1024, scale: float = 8.0, seed: int = 7, amplitude: float = 0.1,
            octaves: int = 6, base_freq: float = 4.0) -> Mesh:
    """Heightfield over the unit square, mapped to world [-scale, scale]^2 (Y up).

    Height = amplitude * fBm(base_freq * (x, z)) in unit coordinates, times 2*scale in world
    space. Cell (i, j) holds triangles (p[i,j], p[i,j+1], p[i+1,j]) and
    (p[i+1,j], p[i,j+1], p[i+1,j+1]), wound so that their face normals point up (+Y), i.e.
    front-facing for rays from above under the reference's one-sided test.
    """
    m = n + 1
    u = (np.arange(m, dtype=np.int64).astype(F) / F(n)).astype(F)
    ux, uz = np.meshgrid(u, u, indexing="ij")
    h = (F(amplitude) * fbm2(ux * F(base_freq), uz * F(base_freq), octaves, seed)).astype(F)
    s2 = F(2.0 * scale)
    wx = (ux - F(0.5)) * s2
    wz = (uz - F(0.5)) * s2
    wy = h * s2
    verts = np.stack([wx.ravel(), wy.ravel(), wz.ravel()], axis=1).astype(F)
    i = np.arange(n, dtype=np.int64)
    ii, jj = np.meshgrid(i, i, indexing="ij")
    p00 = (ii * m + jj).ravel()
    p01 = (ii * m + jj + 1).ravel()
    p10 = ((ii + 1) * m + jj).ravel()
    p11 = ((ii + 1) * m + jj + 1).ravel()
    tris = np.empty((2 * n * n, 3), dtype=np.int32)
    tris[0::2] = np.stack([p00, p01, p10], axis=1)
    tris[1::2] = np.stack([p10, p01, p11], axis=1)
    normals = vertex_normals(verts, tris)
    mat = np.zeros(tris.shape[0], dtype=np.uint32)
    return Mesh(verts, normals, tris, tris.copy(), mat,
                [{"name": "terrain", "type": "Diff", "diffuseColor": [0.7, 0.7, 0.7]}])


_ICO_CACHE: dict[int, tuple[np.ndarray, np.ndarray]] = {}


def icosphere(subdiv: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (vertices float32 (V,3), triangles int32 (T,3)), outward winding."""
    if subdiv in _ICO_CACHE:
        v, t = _ICO_CACHE[subdiv]
        return v.copy(), t.copy()
    phi = F((1.0 + math.sqrt(5.0)) / 2.0)
    o, p = F(1.0), phi
    base = np.array([[-o, p, 0], [o, p, 0], [-o, -p, 0], [o, -p, 0],
                     [0, -o, p], [0, o, p], [0, -o, -p], [0, o, -p],
                     [p, 0, -o], [p, 0, o], [-p, 0, -o], [-p, 0, o]], dtype=F)
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = list(_normalize(base))
    tris = np.array(faces, dtype=np.int64)
    for _ in range(subdiv):
        cache: dict[tuple[int, int], int] = {}
        vs = verts
        new = []

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            idx = cache.get(key)
            if idx is None:
                m = (vs[a] + vs[b]) * F(0.5)
                m = m / np.sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2])
                idx = len(vs)
                vs.append(m.astype(F))
                cache[key] = idx
            return idx

        for a, b, c in tris.tolist():
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        tris = np.array(new, dtype=np.int64)
        verts = vs
    v = np.array(verts, dtype=F)
    t = tris.astype(np.int32)
    _ICO_CACHE[subdiv] = (v, t)
    return v.copy(), t.copy()


def displaced_icosphere(subdiv: int, radius: float, center, seed: int, amplitude: float,
                        freq: float = 4.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Icosphere of `radius` whose vertices move radially by amplitude * value_noise3."""
    v, t = icosphere(subdiv)
    d = value_noise3(v[:, 0] * F(freq), v[:, 1] * F(freq), v[:, 2] * F(freq), seed)
    r = F(radius) + F(amplitude) * d
    verts = (v * r[:, None] + np.asarray(center, dtype=F)[None, :]).astype(F)
    return verts, t, vertex_normals(verts, t)


def _concat(parts: list[tuple[np.ndarray, np.ndarray, np.ndarray, int]]) -> Mesh:
    vs, ns, ts, ms = [], [], [], []
    base = 0
    for verts, tris, normals, mat in parts:
        vs.append(verts)
        ns.append(normals)
        ts.append(tris.astype(np.int64) + base)
        ms.append(np.full(tris.shape[0], mat, dtype=np.uint32))
        base += verts.shape[0]
    tris = np.concatenate(ts).astype(np.int32)
    return Mesh(np.concatenate(vs).astype(F), np.concatenate(ns).astype(F), tris, tris.copy(),
                np.concatenate(ms))


def quad(p0, p1, p2) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Parallelogram p0, p1, p2, p1+p2-p0 as two triangles with face normal (p1-p0)x(p2-p0)."""
    p0, p1, p2 = (np.asarray(p, dtype=F) for p in (p0, p1, p2))
    p3 = p1 + p2 - p0
    verts = np.stack([p0, p1, p2, p3]).astype(F)
    tris = np.array([[0, 1, 2], [2, 1, 3]], dtype=np.int32)
    n = _normalize(_cross((p1 - p0)[None], (p2 - p0)[None]))
    return verts, tris, np.repeat(n, 4, axis=0)


def cornell(subdiv: int = 5, seed: int = 42) -> Mesh:
    """Unit Cornell box (5 walls of 2 triangles, inward-facing) with a 0.25 x 0.25 ceiling
    light and a displaced icosphere of radius 0.3 (amplitude 0.03, seed 42).

    Materials: 0 white 0.73, 1 red (0.65,0.05,0.05), 2 green (0.12,0.45,0.15),
    3 light (emission 17,12,4), 4 sphere Lambert 0.8.
    """
    lo, hi = -0.5, 0.5
    parts = [
        (*quad([lo, lo, lo], [lo, lo, hi], [hi, lo, lo]), 0),   # floor, normal +Y
        (*quad([lo, hi, lo], [hi, hi, lo], [lo, hi, hi]), 0),   # ceiling, normal -Y
        (*quad([lo, lo, lo], [hi, lo, lo], [lo, hi, lo]), 0),   # back wall, normal +Z
        (*quad([lo, lo, lo], [lo, hi, lo], [lo, lo, hi]), 1),   # left wall (red), normal +X
        (*quad([hi, lo, lo], [hi, lo, hi], [hi, hi, lo]), 2),   # right wall (green), normal -X
        (*quad([-0.125, hi - 1e-3, -0.125], [0.125, hi - 1e-3, -0.125], [-0.125, hi - 1e-3, 0.125]), 3),
    ]
    sv, st, sn = displaced_icosphere(subdiv, 0.3, [0.0, -0.2, 0.0], seed, 0.03)
    parts.append((sv, st, sn, 4))
    m = _concat(parts)
    m.materials = [
        {"name": "a_white", "type": "Diff", "diffuseColor": [0.73, 0.73, 0.73]},
        {"name": "b_red", "type": "Diff", "diffuseColor": [0.65, 0.05, 0.05]},
        {"name": "c_green", "type": "Diff", "diffuseColor": [0.12, 0.45, 0.15]},
        {"name": "d_light", "type": "Diff", "diffuseColor": [0.0, 0.0, 0.0], "emission": [17.0, 12.0, 4.0]},
        {"name": "e_sphere", "type": "Diff", "diffuseColor": [0.8, 0.8, 0.8]},
    ]
    return m


def multi_material(count: int = 400, subdiv: int = 5, seed: int = 3, world: float = 4.0) -> Mesh:
    """`count` displaced icospheres (radii U(0.05,0.3), centres uniform in a 10x10x2 box) over
    a 2-triangle ground plane, scaled by `world` (so the smallest sphere stays above the
    reference's 1e-5 determinant cut-off). Material family per sphere: Lambert albedo
    U(0.1,0.9)^3, GGX conductor roughness U(0.05,0.5) and F0 U(0.5,1)^3, or dielectric IOR 1.5.
    Material 0 is the ground (Lambert 0.5); sphere k uses material k+1.
    """
    k = np.arange(count, dtype=np.uint32)
    u = lambda j: hash_uniform(k * np.uint32(16) + np.uint32(j) + np.uint32(seed) * np.uint32(7919))
    radius = (F(0.05) + F(0.25) * u(0)) * F(world)
    cx = (u(1) * F(10.0) - F(5.0)) * F(world)
    cz = (u(2) * F(10.0) - F(5.0)) * F(world)
    cy = (u(3) * F(2.0)) * F(world) + radius
    fam = (pcg_hash(k + np.uint32(seed) * np.uint32(104729)) % np.uint32(3)).astype(np.int64)
    g = F(6.0 * world)
    parts = [(*quad([-g, 0.0, -g], [-g, 0.0, g], [g, 0.0, -g]), 0)]
    materials = [{"name": "m0000_ground", "type": "Diff", "diffuseColor": [0.5, 0.5, 0.5]}]
    for i in range(count):
        verts, tris, normals = displaced_icosphere(subdiv, float(radius[i]), [cx[i], cy[i], cz[i]],
                                                   seed * 1000 + i, 0.1 * float(radius[i]))
        parts.append((verts, tris, normals, i + 1))
        name = f"m{i + 1:04d}"
        if fam[i] == 0:
            materials.append({"name": name, "type": "Diff",
                              "diffuseColor": [float(F(0.1) + F(0.8) * u(4 + c)[i]) for c in range(3)]})
        elif fam[i] == 1:
            materials.append({"name": name, "type": "GGX", "roughness": float(F(0.05) + F(0.45) * u(7)[i]),
                              "F0": [float(F(0.5) + F(0.5) * u(8 + c)[i]) for c in range(3)]})
        else:
            materials.append({"name": name, "type": "Dielectric", "ior": 1.5})
    m = _concat(parts)
    m.materials = materials
    return m


def sky_env(width: int = 2048, height: int = 1024, sun_dir=(0.3, 0.8, 0.52), sun_radiance: float = 5e4,
            sun_diameter_deg: float = 0.5, tint=(0.55, 0.75, 1.0)) -> np.ndarray:
    """Equirectangular sky (h, w, 3) float32 in the reference's mapping (u = atan2(x, z) / 2pi,
    v = acos(y) / pi, row 0 = up): radiance from 0.2 at the horizon to 1.0 at the zenith (times
    a tint), 0.2 below the horizon, plus a sun disc of the given angular diameter and radiance."""
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    theta = v * np.pi
    phi = u * 2.0 * np.pi
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    dx, dy, dz = st * np.sin(phi)[None, :], np.broadcast_to(ct, (height, width)), st * np.cos(phi)[None, :]
    g = 0.2 + 0.8 * np.clip(dy, 0.0, 1.0)
    img = np.stack([g * tint[0], g * tint[1], g * tint[2]], axis=-1)
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    cosang = dx * s[0] + dy * s[1] + dz * s[2]
    disc = cosang >= np.cos(np.radians(sun_diameter_deg / 2.0))
    if not disc.any():  # coarser maps than the disc: light the nearest texel
        disc = cosang == cosang.max()
    img[disc] = sun_radiance
    return img.astype(np.float32)


def material_showcase(subdiv: int = 3) -> tuple["Mesh", list[dict]]:
    """Spheres of every material kind over a ground quad, for the renderer tests: Diff, Metal,
    Spec, Refr, Coat (the reference's kinds), GGX conductor and dielectric. Also returns the
    analytic objects (a Plane backdrop and a Sphere) the JSON scenes can carry."""
    mats = [{"name": "ground", "type": "Diff", "diffuseColor": [0.6, 0.6, 0.6]},
            {"name": "diff", "type": "Diff", "diffuseColor": [0.8, 0.3, 0.2]},
            {"name": "metal", "type": "Metal", "color": [0.9, 0.8, 0.5]},
            {"name": "spec", "type": "Spec", "color": [0.95, 0.95, 0.95]},
            {"name": "refr", "type": "Refr"},
            {"name": "coat", "type": "Coat", "diffuseColor": [0.2, 0.4, 0.8], "specularColor": [0.9, 0.9, 0.9]},
            {"name": "ggx", "type": "GGX", "F0": [0.95, 0.64, 0.54], "roughness": 0.3},
            {"name": "glass", "type": "Dielectric", "ior": 1.5},
            {"name": "lamp", "type": "Diff", "diffuseColor": [0.0, 0.0, 0.0], "emission": [6.0, 6.0, 5.0]}]
    parts = [(*quad([-4.0, 0.0, -4.0], [-4.0, 0.0, 4.0], [4.0, 0.0, -4.0]), 0)]
    for k in range(1, 8):
        x = -2.4 + 0.8 * (k - 1)
        verts, tris, normals = displaced_icosphere(subdiv, 0.35, [x, 0.36, 0.0], 100 + k, 0.0)
        parts.append((verts, tris, normals, k))
    m = _concat(parts)
    m.materials = mats
    geoms = [{"type": "Plane", "p0": [-4.0, 0.0, -1.5], "p1": [4.0, 0.0, -1.5], "p2": [-4.0, 3.0, -1.5],
              "material": 0},
             {"type": "Sphere", "radius": 0.25, "position": [0.0, 1.6, 0.5], "material": 8}]
    return m, geoms


# ---- rays ----------------------------------------------------------------------------------
def pinhole_rays(width: int, height: int, eye, target, tan_half_fov: float,
                 tmin: float = 0.01, tmax: float = 1e20) -> np.ndarray:
    """Primary rays through pixel centres (jitter 0): (W*H, 8) float32, row 0 at the top."""
    eye = np.asarray(eye, dtype=F)
    fwd = _normalize((np.asarray(target, dtype=F) - eye)[None])[0]
    up = np.array([0.0, 1.0, 0.0], dtype=F)
    right = _normalize(_cross(fwd[None], up[None]))[0]
    upv = _cross(right[None], fwd[None])[0]
    aspect = F(width) / F(height)
    xs = ((np.arange(width, dtype=F) + F(0.5)) / F(width) * F(2.0) - F(1.0)) * F(tan_half_fov) * aspect
    ys = (F(1.0) - (np.arange(height, dtype=F) + F(0.5)) / F(height) * F(2.0)) * F(tan_half_fov)
    gx, gy = np.meshgrid(xs, ys, indexing="xy")
    d = (fwd[None, None, :] + gx[..., None] * right[None, None, :] + gy[..., None] * upv[None, None, :])
    d = _normalize(d.reshape(-1, 3).astype(F))
    rays = np.empty((d.shape[0], 8), dtype=F)
    rays[:, 0:3] = eye
    rays[:, 3:6] = d
    rays[:, 6] = F(tmin)
    rays[:, 7] = F(tmax)
    return rays


def _basis(n: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Orthonormal tangents of unit normals n (exact float32 ops, branch on |n.x|)."""
    a = np.where(np.abs(n[:, 0:1]) > F(0.1), np.array([[0, 1, 0]], dtype=F), np.array([[1, 0, 0]], dtype=F))
    t = _normalize(_cross(a, n))
    b = _cross(n, t)
    return t, b


def cosine_hemisphere(normals: np.ndarray, seed: int) -> np.ndarray:
    """Cosine-distributed unit directions about `normals` (Malley: a uniform disk point lifted
    to the hemisphere). The disk point comes from the first of 8 hashed candidates inside the
    unit disk (rejection sampling without transcendentals)."""
    n = normals.shape[0]
    idx = np.arange(n, dtype=np.uint64)
    x = np.zeros(n, dtype=F)
    y = np.zeros(n, dtype=F)
    done = np.zeros(n, dtype=bool)
    for c in range(8):
        key = (idx * np.uint64(16) + np.uint64(2 * c) + np.uint64(seed) * np.uint64(0x9E3779B1)) & np.uint64(0xFFFFFFFF)
        cx = hash_uniform(key.astype(np.uint32)) * F(2.0) - F(1.0)
        cy = hash_uniform((key + np.uint64(1)).astype(np.uint32)) * F(2.0) - F(1.0)
        ok = (~done) & (cx * cx + cy * cy < F(1.0))
        x = np.where(ok, cx, x)
        y = np.where(ok, cy, y)
        done |= ok
    z = np.sqrt(np.maximum(F(0.0), F(1.0) - x * x - y * y)).astype(F)
    t, b = _basis(normals)
    d = t * x[:, None] + b * y[:, None] + normals * z[:, None]
    return _normalize(d.astype(F))


def orbit_views(count: int = 64, seed: int = 5, scale: float = 8.0, sizes=(256, 512, 768, 1024),
                spps=(4, 16, 64), fov: float = 60.0) -> list[tuple]:
    """Camera views for a batched render of the terrain: orbit poses in the reference's camera
    model (eye = centre + (sin yaw cos pitch, sin pitch, cos yaw cos pitch) * radius, looking at the
    centre, src/core/Camera.cpp:121-140) with yaw U[0, 2pi), pitch U(0.25, 0.9) rad and radius
    1.5 * scale; square images of a size drawn from `sizes` and a sample count drawn from `spps`.
    Returns [(tt_camera_meta, spp, sample_offset 0, seed)]."""
    from .core import make_camera_meta

    rng = np.random.default_rng(seed)
    views = []
    for k in range(count):
        yaw = float(rng.uniform(0.0, 2.0 * np.pi))
        pitch = float(rng.uniform(0.25, 0.9))
        res = int(rng.choice(sizes))
        spp = int(rng.choice(spps))
        r = 1.5 * scale
        eye = [r * np.sin(yaw) * np.cos(pitch), r * np.sin(pitch), r * np.cos(yaw) * np.cos(pitch)]
        cam = make_camera_meta(res, res, eye, [-eye[0], -eye[1], -eye[2]], fov=(fov, fov))
        views.append((cam, spp, 0, 1000 + k))
    return views


def terrain_camera(scale: float) -> dict:
    """The recorded pose of the terrain ray-cast benchmark."""
    return {"eye": [0.0, 0.9 * scale, 1.6 * scale], "target": [0.0, 0.0, 0.1 * scale], "tan_half_fov": 0.45}


def secondary_rays(primary: np.ndarray, hit_t: np.ndarray, hit_normal: np.ndarray, count: int,
                   seed: int, tmin: float) -> tuple[np.ndarray, np.ndarray]:
    """`count` incoherent rays: hit pixels resampled (hashed, with replacement), origin at the
    hit point, direction cosine-distributed about the unit hit normal (flipped to face the
    incoming ray). Returns (rays (count, 8), chosen primary indices)."""
    hit = np.nonzero(hit_t < F(1e19))[0]
    if hit.size == 0:
        raise ValueError("no primary hits to spawn secondary rays from")
    k = np.arange(count, dtype=np.uint32)
    pick = hit[(pcg_hash(k ^ np.uint32(seed * 2654435761 & 0xFFFFFFFF)) % np.uint32(hit.size)).astype(np.int64)]
    o = primary[pick, 0:3] + primary[pick, 3:6] * hit_t[pick, None]
    nrm = _normalize(hit_normal[pick].astype(F))
    flip = (nrm * primary[pick, 3:6]).sum(axis=1) > 0
    nrm[flip] = -nrm[flip]
    d = cosine_hemisphere(nrm, seed)
    rays = np.empty((count, 8), dtype=F)
    rays[:, 0:3] = o
    rays[:, 3:6] = d
    rays[:, 6] = F(tmin)
    rays[:, 7] = F(1e20)
    return rays, pick


def shadow_rays(primary: np.ndarray, hit_t: np.ndarray, light, count: int, seed: int,
                tmin: float) -> np.ndarray:
    """`count` shadow rays from hashed primary hit points toward the point `light`;
    tmax = the distance to the light."""
    hit = np.nonzero(hit_t < F(1e19))[0]
    k = np.arange(count, dtype=np.uint32)
    pick = hit[(pcg_hash(k ^ np.uint32((seed * 40503 + 17) & 0xFFFFFFFF)) % np.uint32(hit.size)).astype(np.int64)]
    o = primary[pick, 0:3] + primary[pick, 3:6] * hit_t[pick, None]
    v = np.asarray(light, dtype=F)[None, :] - o
    dist = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2]).astype(F)
    rays = np.empty((count, 8), dtype=F)
    rays[:, 0:3] = o
    rays[:, 3:6] = v / dist[:, None]
    rays[:, 6] = F(tmin)
    rays[:, 7] = dist
    return rays


def random_rays(count: int, seed: int, lo, hi, tmin: float = 0.0) -> np.ndarray:
    """Rays with hashed origins in the box [lo, hi] and hashed directions (normalised
    from a [-1,1]^3 cube sample), for adversarial/unit tests."""
    k = np.arange(count, dtype=np.uint32) * np.uint32(8) + np.uint32(seed) * np.uint32(1000003)
    lo = np.asarray(lo, dtype=F)
    hi = np.asarray(hi, dtype=F)
    o = np.stack([lo[c] + (hi[c] - lo[c]) * hash_uniform(k + np.uint32(c)) for c in range(3)], axis=1)
    d = np.stack([hash_uniform(k + np.uint32(3 + c)) * F(2.0) - F(1.0) for c in range(3)], axis=1)
    d = _normalize(d.astype(F))
    rays = np.empty((count, 8), dtype=F)
    rays[:, 0:3] = o
    rays[:, 3:6] = d
    rays[:, 6] = F(tmin)
    rays[:, 7] = F(1e20)
    return rays


# ---- reference file formats ------------------------------------------------------------------
def write_obj(path: str, mesh: Mesh, mtllib: str) -> None:
    """OBJ with one `vn` per `v`, a `g` group and `mtllib`/`usemtl` per material, as the
    reference's OBJ loader requires. Faces are written `v/t/n` (t unused): the reference's
    face parser never consumes the second slash of `v//n` and loops until memory runs out
    (src/loader/OBJLoader.cpp:70-79)."""
    with open(path, "w") as f:
        f.write(f"mtllib {mtllib}\n")
        for v in mesh.vertices:
            f.write(f"v {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
        for n in mesh.normals:
            f.write(f"vn {float(n[0])!r} {float(n[1])!r} {float(n[2])!r}\n")
        for m in np.unique(mesh.mat):
            f.write(f"g group{int(m)}\nusemtl {mesh.materials[int(m)]['name']}\n")
            for t, nt in zip(mesh.vidx[mesh.mat == m], mesh.nidx[mesh.mat == m]):
                f.write("f " + " ".join(f"{int(a) + 1}/1/{int(b) + 1}" for a, b in zip(t, nt)) + "\n")


def material_json(materials: list[dict]) -> dict:
    return {m["name"]: {k: v for k, v in m.items() if k != "name"} for m in materials}
