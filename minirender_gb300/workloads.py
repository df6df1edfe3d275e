"""Seeded synthetic scenes for the five benchmark configurations plus the
edge cases the parity tests use.

The primitive generators restate src/primitives.cpp (createCube :7-48,
createCylinder :50-148, createSphere :150-230) with numpy; trigonometry is
evaluated in double and rounded once to float32.  Everything here builds
inputs only: the device path and the oracle receive the same arrays.

Configs (sizes as stated in the benchmark definition):
  1  UV sphere 64 slices x 32 stacks, 640x480, point light, Blinn-Phong.
  2  icosphere level 8 (1,310,720 triangles) with value-noise displacement,
     smooth normals, spherical UVs, 1024^2 RGB8 noise+checkerboard texture,
     1920x1080, camera close enough that near-plane clipping runs.
  3  10M-triangle soup, 1-4 px^2 each, depth uniform in [0.2,50], 5% exact
     coplanar duplicates after their originals, per-face colour through a
     palette texture, 3840x2160.
  4  256 scenes x 64 primitives (cube/sphere/cylinder), random TRS
     hierarchy and materials, per-scene resolution and camera.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from . import projection as pj
from .frame import FrameState
from .scene import Material, Scene, SceneNode, TriMesh

f32 = np.float32
PIF = f32(3.14159265)


def _cos(x):
    return np.cos(np.asarray(x, np.float64)).astype(np.float32)


def _sin(x):
    return np.sin(np.asarray(x, np.float64)).astype(np.float32)


def _normalized(v: np.ndarray) -> np.ndarray:
    """Vec3::normalized as float32 ops: v / sqrt(x*x+y*y+z*z)."""
    v = np.asarray(v, np.float32)
    l2 = v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]
    l2 = l2 + v[..., 2] * v[..., 2]
    l = np.sqrt(l2)
    return v / l[..., None]


# ---------------------------------------------------------------- primitives
def create_cube(size: float = 1.0) -> TriMesh:
    """createCube, src/primitives.cpp:7-48."""
    h = f32(size) * f32(0.5)
    faces = [
        ((h, -h, -h), (h, -h, h), (h, h, h), (h, h, -h), (1, 0, 0)),
        ((-h, -h, h), (-h, -h, -h), (-h, h, -h), (-h, h, h), (-1, 0, 0)),
        ((-h, h, -h), (h, h, -h), (h, h, h), (-h, h, h), (0, 1, 0)),
        ((-h, -h, h), (h, -h, h), (h, -h, -h), (-h, -h, -h), (0, -1, 0)),
        ((h, -h, h), (-h, -h, h), (-h, h, h), (h, h, h), (0, 0, 1)),
        ((-h, -h, -h), (h, -h, -h), (h, h, -h), (-h, h, -h), (0, 0, -1)),
    ]
    V, N, T, I = [], [], [], []
    uv = [(0, 0), (1, 0), (1, 1), (0, 1)]
    for f in faces:
        base = len(V)
        V += [f[0], f[1], f[2], f[3]]
        N += [f[4]] * 4
        T += uv
        I += [base + 0, base + 2, base + 1, base + 0, base + 3, base + 2]
    return TriMesh(np.array(V, np.float32), np.array(N, np.float32), np.array(I, np.int32),
                   texcoords=np.array(T, np.float32), material=Material())


def create_cylinder(radius: float, height: float, segments: int = 32, height_segments: int = 1,
                    caps: bool = True) -> TriMesh:
    """createCylinder, src/primitives.cpp:50-148."""
    segments = max(3, segments)
    height_segments = max(1, height_segments)
    radius, height = f32(radius), f32(height)
    half_h = height * f32(0.5)
    two_pi = f32(2.0) * PIF
    V, N, T = [], [], []
    for hh in range(height_segments + 1):
        v = f32(hh) / f32(height_segments)
        z = -half_h + v * height
        u = np.arange(segments, dtype=np.float32) / f32(segments)
        ang = u * two_pi
        x = radius * _cos(ang)
        y = radius * _sin(ang)
        p = np.stack([x, y, np.full_like(x, z)], 1)
        V.append(p)
        N.append(_normalized(np.stack([x, y, np.zeros_like(x)], 1)))
        T.append(np.stack([u, np.full_like(u, v)], 1))
    V = np.concatenate(V)
    N = np.concatenate(N)
    T = np.concatenate(T)
    I = []
    for hh in range(height_segments):
        for r in range(segments):
            i0 = hh * segments + r
            i1 = hh * segments + (r + 1) % segments
            i2 = (hh + 1) * segments + r
            i3 = (hh + 1) * segments + (r + 1) % segments
            I += [i0, i1, i2, i1, i3, i2]
    V, N, T = list(V), list(N), list(T)
    if caps:
        def ring(start_orig, nz):
            ring_start = len(V)
            for r in range(segments):
                p = V[start_orig + r]
                V.append(p.copy())
                N.append(np.array([0, 0, nz], np.float32))
                T.append(np.array([(p[0] / radius + f32(1.0)) * f32(0.5),
                                   (p[1] / radius + f32(1.0)) * f32(0.5)], np.float32))
            return ring_start
        b0 = ring(0, -1)
        bc = len(V)
        V.append(np.array([0, 0, -half_h], np.float32))
        N.append(np.array([0, 0, -1], np.float32))
        T.append(np.array([0.5, 0.5], np.float32))
        for r in range(segments):
            I += [bc, b0 + (r + 1) % segments, b0 + r]
        t0 = ring(height_segments * segments, 1)
        tc = len(V)
        V.append(np.array([0, 0, half_h], np.float32))
        N.append(np.array([0, 0, 1], np.float32))
        T.append(np.array([0.5, 0.5], np.float32))
        for r in range(segments):
            I += [tc, t0 + r, t0 + (r + 1) % segments]
    return TriMesh(np.array(V, np.float32), np.array(N, np.float32), np.array(I, np.int32),
                   texcoords=np.array(T, np.float32), material=Material())


def create_sphere(radius: float, lat_segments: int = 16, long_segments: int = 32) -> TriMesh:
    """createSphere, src/primitives.cpp:150-230."""
    lat_segments = max(2, lat_segments)
    long_segments = max(3, long_segments)
    radius = f32(radius)
    V = [np.array([[0, radius, 0]], np.float32)]
    N = [np.array([[0, 1, 0]], np.float32)]
    T = [np.array([[0.5, 0]], np.float32)]
    u = np.arange(long_segments, dtype=np.float32) / f32(long_segments)
    theta = u * f32(2.0) * PIF
    for lat in range(1, lat_segments):
        v = f32(lat) / f32(lat_segments)
        phi = v * PIF
        sp, cp = _sin(phi), _cos(phi)
        x = radius * sp * _cos(theta)
        y = np.full_like(x, radius * cp)
        z = radius * sp * _sin(theta)
        p = np.stack([x, y, z], 1)
        V.append(p)
        N.append(_normalized(p))
        T.append(np.stack([u, np.full_like(u, f32(1.0) - v)], 1))
    bottom = sum(a.shape[0] for a in V)
    V.append(np.array([[0, -radius, 0]], np.float32))
    N.append(np.array([[0, -1, 0]], np.float32))
    T.append(np.array([[0.5, 1]], np.float32))
    first = 1
    I = []
    L = long_segments
    for lon in range(L):
        I += [0, first + lon, first + (lon + 1) % L]
    rings = lat_segments - 1
    for lat in range(rings - 1):
        r1 = first + lat * L
        r2 = r1 + L
        for lon in range(L):
            a, b = r1 + lon, r1 + (lon + 1) % L
            c, d = r2 + lon, r2 + (lon + 1) % L
            I += [a, b, c, b, d, c]
    last = first + (rings - 1) * L
    for lon in range(L):
        I += [bottom, last + lon, last + (lon + 1) % L]
    return TriMesh(np.concatenate(V), np.concatenate(N), np.array(I, np.int32),
                   texcoords=np.concatenate(T), material=Material())


# ------------------------------------------------------------------ config 1
def config1(width: int = 640, height: int = 480) -> Tuple[FrameState, Scene]:
    """UV sphere, 64 slices x 32 stacks, radius 1, camera at z=4, fov 45,
    near 0.1, far 100, point light (5,5,5), diffuse (0.8,0.5,0.3), specular 1,
    exponent 32, no texture."""
    mesh = create_sphere(1.0, 32, 64)
    mesh.material = Material(diffuse=(0.8, 0.5, 0.3), specular=(1, 1, 1), shininess=32)
    scene = Scene()
    scene.add(mesh)
    st = FrameState(width=width, height=height,
                    projection=pj.projection_frustum(pj.deg2rad(45), f32(width) / f32(height),
                                                     0.1, 100),
                    view=pj.translate(0, 0, -4), light=np.array([5, 5, 5], np.float32),
                    light_is_point=True, ambient=scene.ambientLight)
    return st, scene


# ------------------------------------------------------------------ config 2
_ICO_CACHE = {}


def icosphere(level: int) -> Tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (V,3) float64 positions and (T,3) int32 faces, wound
    so that the reference's edge functions see the outside as front-facing."""
    if level in _ICO_CACHE:
        return _ICO_CACHE[level]
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.stack([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 1)
        e = np.sort(edges.reshape(-1, 2), axis=1)
        key = e[:, 0] * (v.shape[0] + 1) + e[:, 1]
        uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
        ue = e[first]
        mid = (v[ue[:, 0]] + v[ue[:, 1]]) * 0.5
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = (v.shape[0] + inv).reshape(-1, 3)
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        v = np.concatenate([v, mid])
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                            np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    _ICO_CACHE[level] = (v, f.astype(np.int32))
    return _ICO_CACHE[level]


def _hash01(ix, iy, iz, seed):
    """SplitMix64-style hash of integer lattice points to [0,1)."""
    x = (ix.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
         ^ iy.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)
         ^ iz.astype(np.uint64) * np.uint64(0x165667B19E3779F9)
         ^ np.uint64(seed) * np.uint64(0x27D4EB2F165667C5))
    x ^= x >> np.uint64(30)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(27)
    x *= np.uint64(0x94D049BB133111EB)
    x ^= x >> np.uint64(31)
    return (x >> np.uint64(11)).astype(np.float64) / float(1 << 53)


def value_noise(p: np.ndarray, freq: float, seed: int) -> np.ndarray:
    """Trilinear value noise with smoothstep weights, in [0,1]."""
    q = p * freq
    i0 = np.floor(q).astype(np.int64)
    fr = q - i0
    w = fr * fr * (3 - 2 * fr)
    out = np.zeros(p.shape[0])
    with np.errstate(over="ignore"):
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = _hash01(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed)
                    wx = w[:, 0] if dx else 1 - w[:, 0]
                    wy = w[:, 1] if dy else 1 - w[:, 1]
                    wz = w[:, 2] if dz else 1 - w[:, 2]
                    out += h * wx * wy * wz
    return out


def noise_texture(size: int, seed: int, checker: int = 8) -> np.ndarray:
    """size x size RGB8: seeded uniform noise with a checker x checker
    checkerboard overlay."""
    rng = np.random.default_rng(seed)
    noise = rng.integers(0, 256, (size, size, 3), dtype=np.int64)
    cell = max(1, size // checker)
    yy, xx = np.mgrid[0:size, 0:size]
    chk = ((yy // cell + xx // cell) % 2).astype(np.int64)
    tex = noise // 2 + 127 * chk[..., None]
    return np.clip(tex, 0, 255).astype(np.uint8)


def displaced_icosphere(level: int, amplitude: float = 0.05, seed: int = 2, freq: float = 4.0):
    """Positions, smooth normals, spherical UVs and faces of the config-2 mesh."""
    v, f = icosphere(level)
    r = 1.0 + amplitude * (2.0 * value_noise(v, freq, seed) - 1.0)
    p = v * r[:, None]
    fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, f[:, k], fn)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    u = 0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * math.pi)
    vv = np.arccos(np.clip(v[:, 1], -1, 1)) / math.pi
    uv = np.stack([u, vv], 1) * 0.998 + 0.001  # keeps every texel index inside the texture
    return p.astype(np.float32), n.astype(np.float32), uv.astype(np.float32), f


def config2(level: int = 8, width: int = 1920, height: int = 1080, tex_size: int = 1024,
            seed: int = 2) -> Tuple[FrameState, Scene]:
    """Displaced textured icosphere filling most of a 1080p frame; the camera
    is 2.2 from the centre with near = 1.2, so the noise bumps nearest the
    camera pierce the near plane and are clipped (all three cases of
    clipTriangle occur)."""
    p, n, uv, f = displaced_icosphere(level, seed=seed)
    idx = f.reshape(-1)
    mesh = TriMesh(p, n, idx, normalsI=idx, texcoords=uv, texcoordsI=idx,
                   material=Material(texture=noise_texture(tex_size, seed + 1)))
    scene = Scene()
    scene.add(mesh)
    view = pj.mat_mul(pj.mat_mul(pj.translate(0, 0, -2.2), pj.rotate_x(0.35)), pj.rotate_z(0.25))
    st = FrameState(width=width, height=height,
                    projection=pj.projection_frustum(pj.deg2rad(50), f32(width) / f32(height),
                                                     1.2, 100),
                    view=view, light=np.array([-0.3, 0.55, 1.0], np.float32), light_is_point=False,
                    ambient=scene.ambientLight)
    return st, scene


# ------------------------------------------------------------------ config 3
def config3(n_tris: int = 10_000_000, width: int = 3840, height: int = 2160, dup_frac: float = 0.05,
            seed: int = 3, palette: int = 64) -> Tuple[FrameState, Scene]:
    """Triangle soup parallel to the image plane: (1-dup_frac)*n unique
    triangles of 1-4 px^2 at view depth uniform in [0.2, 50], then dup_frac*n
    exact copies (same vertex indices, so bit-identical depth) of earlier
    triangles with a different palette colour."""
    rng = np.random.default_rng(seed)
    n_dup = int(round(n_tris * dup_frac))
    n_u = n_tris - n_dup
    fov = pj.deg2rad(60)
    aspect = f32(width) / f32(height)
    P = pj.projection_frustum(fov, aspect, 0.1, 100)
    cx = rng.uniform(0, width, n_u)
    cy = rng.uniform(0, height, n_u)
    d = rng.uniform(0.2, 50.0, n_u)
    area = rng.uniform(1.0, 4.0, n_u)
    rot = rng.uniform(0, 2 * math.pi, n_u)
    # equilateral triangle of the requested area, vertices clockwise on screen
    # (y down), which the reference's edge functions treat as front-facing.
    s = np.sqrt(4 * area / math.sqrt(3))
    rad = s / math.sqrt(3)
    ang = rot[:, None] - np.array([0, 2 * math.pi / 3, 4 * math.pi / 3])[None, :]
    sx = cx[:, None] + rad[:, None] * np.cos(ang)
    sy = cy[:, None] + rad[:, None] * np.sin(ang)
    xn = 2 * sx / width - 1
    yn = 1 - 2 * sy / height
    vx = xn * d[:, None] / float(P[0, 0])
    vy = yn * d[:, None] / float(P[1, 1])
    vz = -np.broadcast_to(d[:, None], vx.shape)
    verts = np.stack([vx, vy, vz], -1).reshape(-1, 3).astype(np.float32)
    # tilted per-face normals so lighting varies
    nrm = np.stack([rng.normal(0, 0.3, n_u), rng.normal(0, 0.3, n_u), np.ones(n_u)], 1)
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    pal = palette * palette
    uvs = np.stack([(np.arange(pal) % palette + 0.5) / palette,
                    (np.arange(pal) // palette + 0.5) / palette], 1).astype(np.float32)
    col_u = rng.integers(0, pal, n_u)
    src = np.sort(rng.choice(n_u, n_dup, replace=False)) if n_dup else np.zeros(0, np.int64)
    col_d = (col_u[src] + 1 + rng.integers(0, pal - 1, n_dup)) % pal
    tri_v = np.arange(3 * n_u, dtype=np.int64).reshape(-1, 3)
    indices = np.concatenate([tri_v, tri_v[src]]).reshape(-1).astype(np.int32)
    normalsI = np.repeat(np.concatenate([np.arange(n_u), src]), 3).astype(np.int32)
    texI = np.repeat(np.concatenate([col_u, col_d]), 3).astype(np.int32)
    ptex = np.random.default_rng(seed + 1).integers(0, 256, (palette, palette, 3)).astype(np.uint8)
    mesh = TriMesh(verts, nrm, indices, normalsI=normalsI, texcoords=uvs, texcoordsI=texI,
                   material=Material(specular=(0.3, 0.3, 0.3), shininess=8, texture=ptex))
    scene = Scene()
    scene.add(mesh)
    st = FrameState(width=width, height=height, projection=P, view=pj.translate(0, 0, 0),
                    light=np.array([0.2, 0.4, 1.0], np.float32), ambient=scene.ambientLight)
    return st, scene


# ------------------------------------------------------------------ config 4
RESOLUTIONS = [(256, 256), (512, 512), (640, 480), (1280, 720)]


def _random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


_PRIM_CACHE = {}


def _primitive(kind: int, seg: int) -> TriMesh:
    """A TriMesh node sharing the (read-only) arrays of one cached primitive."""
    key = (kind, seg if kind else 0)
    if key not in _PRIM_CACHE:
        if kind == 0:
            _PRIM_CACHE[key] = create_cube(1.0)
        elif kind == 1:
            _PRIM_CACHE[key] = create_sphere(0.6, max(2, seg // 2), seg)
        else:
            _PRIM_CACHE[key] = create_cylinder(0.5, 1.2, seg)
    g = _PRIM_CACHE[key]
    return TriMesh(g.vertices, g.normals, g.indices, normalsI=g.normalsI, texcoords=g.texcoords,
                   texcoordsI=g.texcoordsI if g.texcoordsI.size else None)


def config4_scene(seed: int, n_prims: int = 64, resolution=None) -> Tuple[FrameState, Scene]:
    """One batched-launch scene: a seeded hierarchy of primitives with random
    TRS transforms and Blinn-Phong materials, camera on a radius-12 sphere."""
    rng = np.random.default_rng(1000 + seed)
    scene = Scene()
    nodes: List[SceneNode] = []
    for k in range(n_prims):
        kind = int(rng.integers(0, 3))
        seg = int(rng.integers(8, 65))
        mesh = _primitive(kind, seg)
        sc = rng.uniform(0.2, 2.0)
        m = np.eye(4)
        m[:3, :3] = _random_rotation(rng) * sc
        m[:3, 3] = rng.uniform(-5, 5, 3)
        mesh.transform = m.astype(np.float32)
        mesh.material = Material(diffuse=rng.uniform(0.1, 1.0, 3), specular=rng.uniform(0, 1, 3),
                                 emissive=rng.uniform(0, 0.1, 3),
                                 shininess=float(rng.choice([0.0, 4.0, 16.0, 64.0])))
        parent = scene if (k == 0 or rng.uniform() < 0.75) else nodes[int(rng.integers(0, k))]
        parent.add(mesh)
        nodes.append(mesh)
    if resolution is None:
        resolution = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
    w, h = resolution
    d = rng.normal(size=3)
    eye = 12.0 * d / np.linalg.norm(d)
    st = FrameState(width=w, height=h,
                    projection=pj.projection_frustum(pj.deg2rad(50), f32(w) / f32(h), 0.5, 100),
                    view=pj.look_at(eye), light=np.array([-0.3, 0.55, 1.0], np.float32),
                    ambient=scene.ambientLight)
    return st, scene


def config4(n_scenes: int = 256, n_prims: int = 64):
    return [config4_scene(s, n_prims) for s in range(n_scenes)]


# ------------------------------------------------------------------ config 5
def config5_pool(n_meshes: int = 24, seed: int = 5, t_min: int = 1000, t_max: int = 2_000_000):
    """Meshes for the serving stream: config-3 style soups whose triangle
    counts are log-uniform in [t_min, t_max]; each with its palette texture."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(t_min), math.log(t_max), n_meshes)).astype(int)
    pool = []
    for k, n in enumerate(sizes):
        st, sc = config3(n_tris=int(n), width=3840, height=2160, seed=seed * 1000 + k)
        pool.append(sc.children[0])
    return pool


def config5_requests(pool, n: int, rate: float, seed: int = 7, rerender: float = 0.3, key_base: int = 1):
    """A Poisson request stream: arrival times (s), resolution log-uniform
    from 128x128 to 3840x2160, a fresh mesh key (the mesh must be uploaded)
    or, with probability `rerender`, a recently used key re-rendered from a
    new camera.  Fresh keys count up from key_base (give each stream its own
    range so that no key of an earlier stream is found resident)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    out = []
    recent: List[Tuple[int, int]] = []
    next_key = key_base
    for i in range(n):
        u = rng.uniform()
        w = int(round(128 * (3840 / 128) ** u))
        h = int(round(128 * (2160 / 128) ** u))
        if recent and rng.uniform() < rerender:
            key, idx = recent[int(rng.integers(0, len(recent)))]
            angle = float(rng.uniform(-0.3, 0.3))
        else:
            idx = int(rng.integers(0, len(pool)))
            key = next_key
            next_key += 1
            angle = 0.0
            recent.append((key, idx))
            recent = recent[-32:]
        st = FrameState(width=w, height=h,
                        projection=pj.projection_frustum(pj.deg2rad(60), f32(w) / f32(h), 0.1, 100),
                        view=pj.rotate_z(angle), light=np.array([0.2, 0.4, 1.0], np.float32))
        out.append({"t": float(t[i]), "state": st, "mesh": idx, "key": key})
    return out
