"""Procedural scenes and the trace-step workloads.

The reference ships only two usable meshes (objs/icos.obj, objs/smol_menger.obj)
and builds its scenes in Julia scripts (src/scenes/*.jl).  The workloads here
are seeded procedural stand-ins with the sizes the benchmarks are quoted on:

* ``plain_small``   -- icosphere subdivision 5 (10,242 verts / 20,480 tris),
  radius 1, over a 2-triangle diffuse floor at y = -1.5; one directional
  RectLight, 256 x 256 rays, one uniform wavelength per ray, depth 3,
  brute-force hitter, 256 x 256 Float32 light map.
* ``realtime``      -- radially displaced icosphere subdivision 6 (40,962
  verts / 81,920 tris, value-noise amplitude 0.05) over the floor; 2^20
  traced rays (2048 x 2048 light grid, forward upscale 2 so every ray is
  splatted at 2 x 2 footprint offsets through its position Jacobian), 16
  stratified wavelengths, depth 4, BVH hitter, 1024 x 1024 x 16 int32
  fixed-point light map (scale 2^16).
* ``menger``        -- Menger sponge level 3 (8,000 cubes, 96,000 tris) of
  glass rotated by a seeded quaternion inside a 12-triangle diffuse box;
  2^22 rays, 8 wavelengths, depth 6, 2048 x 2048 x 8 map.

Triangle arrays follow the reference layout: ``(T, 10, 3)`` float32 FTri
records, index 0 (reference index 1) the all-zero sentinel, glass triangles
first and diffuse triangles from ``first_diffuse`` (1-based) on, as the
reference's scenes arrange them (src/scenes/sphere.jl:36-37).
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Sequence, Optional

import numpy as np

from . import types as T

# --------------------------------------------------------------------------
# meshes (float64 construction, float32 records)
# --------------------------------------------------------------------------


def _normalize(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def icosphere(subdiv: int):
    """Vertices (unit sphere) and CCW faces of a subdivided icosahedron."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = np.array(
        [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
         (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)],
        dtype=np.float64,
    )
    faces = np.array(
        [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)],
        dtype=np.int64,
    )
    V = _normalize(verts)
    F = faces
    for _ in range(subdiv):
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        e = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 0)
        e = np.sort(e, axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = _normalize(0.5 * (V[uniq[:, 0]] + V[uniq[:, 1]]))
        nf = F.shape[0]
        mab, mbc, mca = (inv[:nf] + len(V), inv[nf:2 * nf] + len(V), inv[2 * nf:] + len(V))
        V = np.concatenate([V, mid], 0)
        F = np.concatenate(
            [np.stack([a, mab, mca], 1), np.stack([b, mbc, mab], 1),
             np.stack([c, mca, mbc], 1), np.stack([mab, mbc, mca], 1)], 0)
    return V, F


def value_noise(p: np.ndarray, freq: float, seed: int) -> np.ndarray:
    """Seeded 3-D value noise in [-1, 1]: random lattice values, smoothstep
    trilinear interpolation."""
    rng = np.random.default_rng(seed)
    n = 64
    lattice = rng.uniform(-1.0, 1.0, size=(n, n, n))
    q = p * freq + n / 2
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    w = f * f * (3.0 - 2.0 * f)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wt = ((w[:, 0] if dx else 1 - w[:, 0]) * (w[:, 1] if dy else 1 - w[:, 1])
                      * (w[:, 2] if dz else 1 - w[:, 2]))
                out += wt * lattice[(i0[:, 0] + dx) % n, (i0[:, 1] + dy) % n, (i0[:, 2] + dz) % n]
    return out


def vertex_normals(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    fn = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    acc = np.zeros_like(V)
    for k in range(3):
        np.add.at(acc, F[:, k], fn)
    return _normalize(acc)


def ftri_records(P: np.ndarray, N: np.ndarray, UV: np.ndarray) -> np.ndarray:
    """Pack per-corner positions / normals / uvs ``(T, 3, 3)`` into FTri
    records.  The plane normal is ``cross(v1 - v2, v2 - v3)`` in binary32, as
    mesh_to_FTri computes it (src/geo.jl:331-341)."""
    P = P.astype(np.float32)
    v1, v2, v3 = P[:, 0], P[:, 1], P[:, 2]
    a = v1 - v2
    b = v2 - v3
    n = np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                  a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                  a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1).astype(np.float32)
    out = np.zeros((P.shape[0], 10, 3), dtype=np.float32)
    out[:, 0] = n
    out[:, 1:4] = P
    out[:, 4:7] = N.astype(np.float32)
    out[:, 7:10] = UV.astype(np.float32)
    return out


def sphere_tris(subdiv: int, radius: float = 1.0, noise_amp: float = 0.0, noise_seed: int = 3,
                center=(0.0, 0.0, 0.0)) -> np.ndarray:
    V, F = icosphere(subdiv)
    if noise_amp:
        V = V * (1.0 + noise_amp * value_noise(V, 3.0, noise_seed))[:, None]
    V = V * radius + np.asarray(center, dtype=np.float64)
    N = vertex_normals(V, F) if noise_amp else _normalize(V - np.asarray(center))
    P = V[F]
    NN = N[F]
    UV = np.zeros_like(P)
    return ftri_records(P, NN, UV)


def floor_tris(y: float = -1.5, half: float = 4.0) -> np.ndarray:
    c = np.array([[-half, y, -half], [half, y, -half], [half, y, half], [-half, y, half]])
    P = np.stack([c[[0, 2, 1]], c[[0, 3, 2]]], 0)
    N = np.zeros_like(P)
    N[..., 1] = 1.0
    UV = np.zeros_like(P)
    UV[..., 0] = (P[..., 0] + half) / (2 * half)
    UV[..., 1] = (P[..., 2] + half) / (2 * half)
    return ftri_records(P, N, UV)


_CUBE_FACES = [  # (normal axis, sign) -> 4 corners (unit cube) CCW seen from outside
    ((0, 0, -1), [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0)]),
    ((0, 0, 1), [(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]),
    ((0, -1, 0), [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)]),
    ((0, 1, 0), [(0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)]),
    ((-1, 0, 0), [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)]),
    ((1, 0, 0), [(1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)]),
]


def _cube_corner_tris():
    P, N = [], []
    for n, q in _CUBE_FACES:
        q = np.asarray(q, dtype=np.float64)
        P += [q[[0, 1, 2]], q[[0, 2, 3]]]
        N += [np.tile(n, (3, 1))] * 2
    return np.asarray(P), np.asarray(N, dtype=np.float64)


def menger_cubes(level: int) -> np.ndarray:
    n = 3 ** level
    idx = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    keep = np.ones(len(idx), dtype=bool)
    d = idx.copy()
    for _ in range(level):
        ones = (d % 3 == 1).sum(1)
        keep &= ones < 2
        d //= 3
    return idx[keep]


def random_quaternion_matrix(seed: int) -> np.ndarray:
    """Uniform random rotation (Shoemake's subgroup algorithm)."""
    u1, u2, u3 = np.random.default_rng(seed).uniform(size=3)
    q = np.array([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def menger_tris(level: int, size: float = 2.0, rotation_seed: Optional[int] = 4) -> np.ndarray:
    cubes = menger_cubes(level)
    s = size / 3 ** level
    Pc, Nc = _cube_corner_tris()
    P = (-size / 2 + (cubes[:, None, None, :] + Pc[None]) * s).reshape(-1, 3, 3)
    N = np.broadcast_to(Nc[None], (len(cubes),) + Nc.shape).reshape(-1, 3, 3)
    if rotation_seed is not None:
        R = random_quaternion_matrix(rotation_seed)
        P = P @ R.T
        N = N @ R.T
    return ftri_records(P, N, np.zeros_like(P))


def box_tris(half: float = 3.0) -> np.ndarray:
    """12 inward-facing triangles; texture atlas of 3 x 2 face cells."""
    Pc, Nc = _cube_corner_tris()
    P = (Pc - 0.5) * 2 * half
    N = -Nc
    UV = np.zeros_like(P)
    for f in range(6):
        axis = int(np.nonzero(Nc[2 * f, 0])[0][0])
        a1, a2 = [k for k in range(3) if k != axis]
        cx, cy = f % 3, f // 3
        for t in (2 * f, 2 * f + 1):
            loc = Pc[t]
            UV[t, :, 0] = (cx + loc[:, a1]) / 3.0
            UV[t, :, 1] = (cy + loc[:, a2]) / 2.0
    P = P[:, ::-1]  # reverse winding: normals point into the box
    N = N[:, ::-1]
    UV = UV[:, ::-1]
    return ftri_records(P, N, UV)


def assemble(glass: np.ndarray, diffuse: np.ndarray):
    """Sentinel + glass + diffuse; returns (tris, first_diffuse 1-based)."""
    sentinel = np.zeros((1, 10, 3), dtype=np.float32)
    tris = np.concatenate([sentinel, glass, diffuse], 0).astype(np.float32)
    return np.ascontiguousarray(tris), 1 + glass.shape[0] + 1


# --------------------------------------------------------------------------
# lights and workloads
# --------------------------------------------------------------------------


def hemisphere_light(seed: int, res: int, aperture: float, distance: float = 3.0, min_elev: float = 0.5):
    rng = np.random.default_rng(seed)
    y = rng.uniform(min_elev, 1.0)
    phi = rng.uniform(0.0, 2 * np.pi)
    u = np.array([np.sqrt(1 - y * y) * np.cos(phi), y, np.sqrt(1 - y * y) * np.sin(phi)])
    e = np.array([0.0, 0.0, 1.0]) if abs(u[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    d1 = _normalize(np.cross(u, e))
    d2 = np.cross(u, d1)
    return T.rect_light(distance * u, -u, aperture * d1, aperture * d2, res, res)


@dataclass
class Workload:
    name: str
    tris: np.ndarray
    first_diffuse: int
    light: np.ndarray
    upscale: int = 1
    lambda_mode: tuple = (T.LAMBDA_FIXED, 1, 550.0, 550.0)  # (mode, n_strata, l0, l1)
    spectrum: Optional[np.ndarray] = None  # None: each ray splats at its own wavelength
    depth: int = 3
    material: tuple = (T.MATERIAL_LINEAR_REF, 0.0, 0.0)
    map_w: int = 256
    map_h: int = 256
    accum: str = "f32"  # "f32" float atomics or "i32" fixed point
    frac_bits: int = 16
    hitter: str = "brute"
    seed: int = 2
    force_rand: Optional[float] = None
    quirks: bool = True
    extra: dict = field(default_factory=dict)

    @property
    def n_rays(self) -> int:
        return int(self.light["res1"] // self.upscale) * int(self.light["res2"] // self.upscale)

    @property
    def n_planes(self) -> int:
        return 1 if self.spectrum is None else int(len(self.spectrum))

    @property
    def n_tris(self) -> int:
        return int(self.tris.shape[0])

    def with_(self, **kw) -> "Workload":
        return replace(self, **kw)


CAUCHY_GLASS = (T.MATERIAL_CAUCHY, 1.5, 0.004)


def stratified_spectrum(n: int, lo: float = 400.0, hi: float = 700.0) -> np.ndarray:
    w = np.float32((hi - lo) / n)
    return (np.float32(lo) + (np.arange(n, dtype=np.float32) + np.float32(0.5)) * w).astype(np.float32)


def plain_small(**kw) -> Workload:
    tris, fd = assemble(sphere_tris(5), floor_tris(-1.5, 4.0))
    w = Workload(
        name="icosphere5-20480tris-65536rays-depth3-brute-256x256-f32",
        tris=tris, first_diffuse=fd, light=hemisphere_light(1, 256, 1.05), upscale=1,
        lambda_mode=(T.LAMBDA_UNIFORM, 1, 400.0, 700.0), spectrum=None, depth=3,
        material=CAUCHY_GLASS, map_w=256, map_h=256, accum="f32", hitter="brute", seed=2,
    )
    return w.with_(**kw) if kw else w


def realtime(**kw) -> Workload:
    tris, fd = assemble(sphere_tris(6, noise_amp=0.05, noise_seed=3), floor_tris(-1.5, 4.0))
    w = Workload(
        name="displaced-icosphere6-81920tris-2^20rays-16lambda-depth4-bvh-1024x1024-i32",
        tris=tris, first_diffuse=fd, light=hemisphere_light(1, 2048, 1.1), upscale=2,
        lambda_mode=(T.LAMBDA_STRATIFIED, 16, 400.0, 700.0), spectrum=stratified_spectrum(16), depth=4,
        material=CAUCHY_GLASS, map_w=1024, map_h=1024, accum="i32", hitter="bvh", seed=2,
    )
    return w.with_(**kw) if kw else w


def menger(**kw) -> Workload:
    tris, fd = assemble(menger_tris(3, 2.0, 4), box_tris(3.0))
    light = T.rect_light((0.0, 2.6, 0.0), (0.0, -1.0, 0.0), (1.3, 0.0, 0.0), (0.0, 0.0, 1.3), 2048, 2048)
    w = Workload(
        name="menger3-96000tris-box-2^22rays-8lambda-depth6-bvh-2048x2048-i32",
        tris=tris, first_diffuse=fd, light=light, upscale=1,
        lambda_mode=(T.LAMBDA_STRATIFIED, 8, 400.0, 700.0), spectrum=stratified_spectrum(8), depth=6,
        material=CAUCHY_GLASS, map_w=2048, map_h=2048, accum="i32", hitter="bvh", seed=2,
    )
    return w.with_(**kw) if kw else w


def scaled_light(light: np.ndarray, res: int) -> np.ndarray:
    out = light.copy()
    out["res1"] = res
    out["res2"] = res
    return out


# --------------------------------------------------------------------------
# batched and served workloads
# --------------------------------------------------------------------------


def _loguniform(rng, lo, hi):
    return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def mixed_glass(n_tris: int, seed: int):
    """A glass mesh of exactly n_tris triangles: the smallest displaced
    icosphere or Menger sponge level with at least n_tris triangles, cut to
    n_tris (a seeded choice between the two; Menger only up to level 3).
    Returns (glass tris, 'sphere' | 'menger')."""
    rng = np.random.default_rng(seed)
    if rng.uniform() < 0.5 and n_tris <= 96000:
        level = next(l for l in (1, 2, 3) if 12 * 20 ** l >= n_tris)
        return menger_tris(level, 2.0, rotation_seed=seed)[:n_tris], "menger"
    k = next(k for k in range(1, 9) if 20 * 4 ** k >= n_tris)
    return sphere_tris(k, noise_amp=0.05, noise_seed=seed)[:n_tris], "sphere"


def batched_frames(n: int = 64, seed: int = 5) -> list:
    """Independent frames of uneven size: triangles log-uniform in
    [500, 200000], rays log-uniform in [2^14, 2^22], depth 2..6, 1..16
    wavelength planes, map side log-uniform in [256, 2048], int32 maps."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        n_t = int(round(_loguniform(rng, 500, 200000)))
        rays = _loguniform(rng, 2 ** 14, 2 ** 22)
        res = max(128, int(round(np.sqrt(rays))))
        depth = int(rng.integers(2, 7))
        planes = int(rng.integers(1, 17))
        side = int(round(_loguniform(rng, 256, 2048)))
        glass, kind = mixed_glass(n_t, seed * 1000 + i)
        if kind == "menger":
            tris, fd = assemble(glass, box_tris(3.0))
            light = T.rect_light((0.0, 2.6, 0.0), (0.0, -1.0, 0.0), (1.3, 0.0, 0.0), (0.0, 0.0, 1.3), res, res)
        else:
            tris, fd = assemble(glass, floor_tris(-1.5, 4.0))
            light = hemisphere_light(seed * 1000 + i, res, 1.1)
        out.append(Workload(
            name=f"batch{i}-{kind}-{n_t}tris-{res * res}rays-d{depth}-{planes}l-{side}",
            tris=tris, first_diffuse=fd, light=light, upscale=1,
            lambda_mode=(T.LAMBDA_STRATIFIED, planes, 400.0, 700.0), spectrum=stratified_spectrum(planes),
            depth=depth, material=CAUCHY_GLASS, map_w=side, map_h=side, accum="i32", hitter="bvh",
            seed=seed * 7919 + i))
    return out


def served_scene(sid: int):
    """Scene sid of the serving pool: a level-3 Menger sponge (96,000
    triangles) rotated by a seeded quaternion, in the 12-triangle box."""
    return assemble(menger_tris(3, 2.0, rotation_seed=100 + sid), box_tris(3.0))


def served_request(rng, scene, first_diffuse: int, rid: int) -> Workload:
    """Per-request parameters: light direction perturbed by up to 5 degrees,
    rays / map / depth / planes drawn like the batched frames."""
    rays = _loguniform(rng, 2 ** 14, 2 ** 22)
    res = max(128, int(round(np.sqrt(rays))))
    depth = int(rng.integers(2, 7))
    planes = int(rng.integers(1, 17))
    side = int(round(_loguniform(rng, 256, 2048)))
    ang = np.radians(5.0) * np.sqrt(rng.uniform())
    phi = rng.uniform(0, 2 * np.pi)
    d = np.array([np.sin(ang) * np.cos(phi), -np.cos(ang), np.sin(ang) * np.sin(phi)])
    e = np.array([1.0, 0.0, 0.0])
    d1 = _normalize(np.cross(d, np.array([0.0, 0.0, 1.0])))
    d2 = np.cross(d, d1)
    light = T.rect_light((0.0, 2.6, 0.0), d, 1.3 * d1, 1.3 * d2, res, res)
    del e
    return Workload(name=f"req{rid}", tris=scene, first_diffuse=first_diffuse, light=light, upscale=1,
                    lambda_mode=(T.LAMBDA_STRATIFIED, planes, 400.0, 700.0), spectrum=stratified_spectrum(planes),
                    depth=depth, material=CAUCHY_GLASS, map_w=side, map_h=side, accum="i32", hitter="bvh",
                    seed=1000003 + rid)


# -------------------------------------------------------------------------- camera pass
def realtime_camera() -> dict:
    """A view of the realtime scene (sphere at the origin over the floor at
    y = -1.5), 45-degree field of view (src/scenes/sphere.jl:55-62 style)."""
    return {"pos": (0.0, 2.5, 5.0), "look_at": (0.0, -0.5, 0.0), "up": (0.0, 1.0, 0.0), "fov": 45.0 * np.pi / 180.0}


def gradient_sky(w: int = 512, h: int = 256, seed: int = 6) -> np.ndarray:
    """Procedural skydome [w, h, 3] float32 in [0, 1] (the reference loads
    objs/skydome2.png, which it does not ship): a vertical gradient with seeded
    value-noise clouds."""
    u = (np.arange(w, dtype=np.float64) + 0.5) / w  # polar angle / pi
    v = (np.arange(h, dtype=np.float64) + 0.5) / h  # azimuth
    U, Vv = np.meshgrid(u, v, indexing="ij")
    pts = np.stack([U * 8.0, Vv * 16.0, np.zeros_like(U)], axis=-1).reshape(-1, 3)
    cloud = value_noise(pts, 1.0, seed).reshape(w, h)
    sky = np.zeros((w, h, 3), dtype=np.float32, order="F")
    sky[:, :, 0] = 0.25 + 0.5 * U + 0.2 * cloud
    sky[:, :, 1] = 0.45 + 0.35 * U + 0.2 * cloud
    sky[:, :, 2] = 0.9 - 0.3 * U + 0.1 * cloud
    return np.clip(sky, 0.0, 1.0)


def checkered_map(pixels_per_square: int, squares: int, planes: int, value: float = 12.0) -> np.ndarray:
    """checkered_tex(pixels_per_square, squares, planes) .* value
    (src/procedural_assets.jl:86-97, src/scenes/sphere.jl:43): [w, h, planes]
    float32, w = h = 2 pixels_per_square squares."""
    x = np.tile(np.concatenate([np.ones(pixels_per_square), np.zeros(pixels_per_square)]), squares)
    t = (x[:, None] + x[None, :]) % 2
    out = np.zeros((len(x), len(x), planes), dtype=np.float32, order="F")
    out[:, :, :] = (t * value)[:, :, None]
    return out


# -------------------------------------------------------------------------- mesh ingest
def load_obj(path: str) -> np.ndarray:
    """A Wavefront OBJ file as FTri records (T, 10, 3) through libsplat's
    parser (mesh_to_FTri, src/geo.jl:330-341); no sentinel."""
    import ctypes as C

    from . import _lib as L

    lib = L.load()
    n = C.c_int64()
    L.check(lib.splat_obj_to_ftri(path.encode(), None, 0, C.byref(n)))
    out = np.zeros((n.value, 10, 3), dtype=np.float32)
    L.check(lib.splat_obj_to_ftri(path.encode(), out.ctypes.data, n.value, C.byref(n)))
    return out


def write_obj(path: str, P: np.ndarray, N: np.ndarray, UV: np.ndarray) -> None:
    """Per-corner positions / normals / uvs (T, 3, 3) as an OBJ file with
    shortest round-trip binary32 decimals (one v / vn / vt per corner)."""
    def f(x):
        return repr(float(np.float32(x)))

    with open(path, "w") as fh:
        fh.write("# written by splat_gb300.scenes.write_obj\n")
        for t in range(P.shape[0]):
            for k in range(3):
                fh.write("v %s %s %s\n" % tuple(f(c) for c in P[t, k]))
                fh.write("vn %s %s %s\n" % tuple(f(c) for c in N[t, k]))
                fh.write("vt %s %s\n" % (f(UV[t, k, 0]), f(UV[t, k, 1])))
        for t in range(P.shape[0]):
            a = 3 * t + 1
            fh.write(f"f {a}/{a}/{a} {a + 1}/{a + 1}/{a + 1} {a + 2}/{a + 2}/{a + 2}\n")


def assemble_meshes(glass: Sequence[np.ndarray], diffuse: Sequence[np.ndarray]):
    """The reference's scene layout (src/scenes/sphere.jl:36-38): the zero
    sentinel, then the glass meshes, then the diffuse ones; returns (tris,
    first_diffuse 1-based)."""
    g = np.concatenate(list(glass), 0) if glass else np.zeros((0, 10, 3), np.float32)
    d = np.concatenate(list(diffuse), 0) if diffuse else np.zeros((0, 10, 3), np.float32)
    return assemble(g, d)


def translate(tris: np.ndarray, offset) -> np.ndarray:
    """translate(t::FTri, v) (src/geo.jl:132-135): vertices moved, normals and uvs kept."""
    out = tris.copy()
    out[:, 1:4] = (out[:, 1:4] + np.asarray(offset, np.float32)).astype(np.float32)
    return out


def scale(tris: np.ndarray, s: float) -> np.ndarray:
    """scale(t::FTri, s) (src/geo.jl:137-138): vertices scaled; the plane
    normal, vertex normals and uvs kept."""
    out = tris.copy()
    out[:, 1:4] = (out[:, 1:4] * np.float32(s)).astype(np.float32)
    return out


def rotate(tris: np.ndarray, R) -> np.ndarray:
    """rotate(t::FTri, R) (src/geo.jl:139-150): plane normal, vertices and
    vertex normals multiplied by the 3 x 3 matrix R; uvs kept."""
    out = tris.copy()
    R = np.asarray(R, np.float32)
    out[:, 0:7] = np.einsum("ij,tkj->tki", R, out[:, 0:7]).astype(np.float32)
    return out


def _ftri(n, a, b, c, na, nb, nc, ta, tb, tc) -> np.ndarray:
    return np.stack([n, a, b, c, na, nb, nc, ta, tb, tc], 1).astype(np.float32)


def _cross32(u: np.ndarray, v: np.ndarray) -> np.ndarray:
    u, v = u.astype(np.float32), v.astype(np.float32)
    return np.stack([u[:, 1] * v[:, 2] - u[:, 2] * v[:, 1], u[:, 2] * v[:, 0] - u[:, 0] * v[:, 2],
                     u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0]], 1).astype(np.float32)


def square() -> np.ndarray:
    """square() (src/procedural_assets.jl:76-84): the unit square at z = 0 as
    two triangles facing +z, uv = position."""
    a, b, c, d = (np.array(v, np.float32)[None] for v in ((0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)))
    n = np.array([[0, 0, 1]], np.float32)
    return np.concatenate([_ftri(n, a, b, c, n, n, n, a, b, c), _ftri(n, b, c, d, n, n, n, b, c, d)], 0)


def stage() -> np.ndarray:
    """stage() (src/procedural_assets.jl:1-18): a floor triangle at z = -2
    and two walls meeting at (0, -2, 2), flat-shaded."""
    p = lambda *v: np.array([v], np.float32)  # noqa: E731
    a, b, c, d = p(3, 1, -2), p(-3, 1, -2), p(0, -2, -2), p(0, -2, 2)
    ta, tb, tc, td = p(0, 0, 0), p(1, 0, 0), p(0.5, 0.5, 0), p(0.5, 1, 0)

    def unit(v):
        return (v / np.sqrt((v.astype(np.float32) ** 2).sum(1, keepdims=True))).astype(np.float32)

    n1 = unit(_cross32(a - b, a - c))
    n2 = unit(_cross32(d - b, d - c))
    n3 = unit(_cross32(d - a, d - c))
    return np.concatenate([_ftri(n1, a, b, c, n1, n1, n1, ta, tb, tc), _ftri(n2, b, c, d, n2, n2, n2, tb, tc, td),
                           _ftri(n3, a, d, c, n3, n3, n3, ta, td, tc)], 0)


def ripples(t: float = 0.0, step: float = 0.005) -> np.ndarray:
    """ripples(t) (src/procedural_assets.jl:20-73): a water surface over the
    unit square, height f(x, y) = (s(50, x) + s(60, x) + s(70, y) + s(80, y))
    * 1.25e-4 with s(k, u) = sin(k u - k tanh(k) t), two triangles per grid
    cell, vertex normals (df/dx, df/dy, -1), uv = (x, y, 0).  The values are
    evaluated in binary64 and stored as binary32; the order of the triangles
    is the reference's (per grid row y, the first triangles of every x, then
    the second ones)."""
    n = int(round(1.0 / step))
    x = np.arange(n, dtype=np.float64) * step
    om = lambda k: k * np.tanh(k)  # noqa: E731

    def f(x, y):
        s = lambda k, u: np.sin(k * u - om(k) * t)  # noqa: E731
        return (s(50, x) + s(60, x) + s(70, y) + s(80, y)) * 0.000125

    def nrm(x, y):
        c = lambda k, u: np.cos(k * u - om(k) * t) * k  # noqa: E731
        return np.stack([(c(50, x) + c(60, x)) * 0.000125, (c(70, y) + c(80, y)) * 0.000125,
                         -np.ones_like(x)], -1).astype(np.float32)

    def vert(x, y):
        return np.stack([x, y, f(x, y)], -1).astype(np.float32)

    X, Y = np.meshgrid(x, x, indexing="xy")  # rows: y, columns: x
    X, Y = X.reshape(-1), Y.reshape(-1)
    dx = dy = step

    def tri(pa, pb, pc):
        a, b, c = vert(*pa), vert(*pb), vert(*pc)
        ta, tb, tc = (np.stack([v[:, 0], v[:, 1], np.zeros_like(v[:, 0])], 1) for v in (a, b, c))
        return _ftri(_cross32(a - b, a - c), a, b, c, nrm(*pa), nrm(*pb), nrm(*pc), ta, tb, tc)

    t1 = tri((X, Y), (X + dx, Y), (X, Y + dy)).reshape(n, n, 10, 3)
    t2 = tri((X + dx, Y + dy), (X + dx, Y), (X, Y + dy)).reshape(n, n, 10, 3)
    return np.ascontiguousarray(np.concatenate([t1, t2], 1).reshape(-1, 10, 3))


def ripples_scene(t: float = 0.0, **kw) -> Workload:
    """The reference's ripples scene (src/scenes/ripples.jl:21-32): the water
    surface (glass) centred on the origin over the unit square three units
    below it (diffuse), lit from above; 80,000 water triangles.  Caustics of
    a moving surface: ripples_scene(t) at successive t are the frames of an
    animation."""
    rips = translate(ripples(t), (-0.5, -0.5, 0.0))
    sq = translate(square(), (-0.5, -1.0, -3.0))
    tris, fd = assemble_meshes([rips], [sq])
    light = T.rect_light((0.0, 0.0, 2.0), (0.0, 0.0, -1.0), (0.6, 0.0, 0.0), (0.0, 0.6, 0.0), 1024, 1024)
    w = Workload(name="ripples-80000tris-2^20rays-depth2-bvh-512x512-i32", tris=tris, first_diffuse=fd, light=light,
                 upscale=1, lambda_mode=(T.LAMBDA_STRATIFIED, 8, 400.0, 700.0), spectrum=stratified_spectrum(8),
                 depth=2, material=(T.MATERIAL_CAUCHY, 1.33, 0.003), map_w=512, map_h=512, accum="i32",
                 hitter="bvh", seed=31)
    return w.with_(**kw) if kw else w
