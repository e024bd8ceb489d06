"""Synthetic scene generators for the workloads the renderer is measured on.

All geometry is float32 triangles ``[n, 3, 3]`` wound so that the DumbRay outward normal
``(c - a) x (b - a)`` (``Triangle::normal()``, __source__/DataStructures/Primitives/Compound/
Triangle/Triangle.impl.h:233-235) points out of closed solids and toward the open side of quads;
that is the side the reference's backface culling keeps visible.

Workloads (no public dataset is involved; every input is generated from a seed):
  * ``box_and_icosphere``       - 12-triangle 2x2x2 box + icosphere level 5 (20,480 tris, r 0.6)
                                  + one 0.5x0.5 emissive quad; 256x256, 16 spp, depth 4.
  * ``displaced_icosphere``     - icosphere level 8 (1,310,720 tris) radially displaced by 3-octave
                                  value noise (amplitude 0.1, seed 1): the ray-cast microbenchmark mesh.
  * ``full_scene``              - the displaced mesh + a 2-triangle ground plane + 4 emissive quads,
                                  materials chosen by a hash of the triangle index.
  * ``batch_workload``          - 64 independent scenes (triangle counts log-uniform 1k-2M: a displaced
                                  icosphere plus random boxes), resolutions from {128..1024}^2, spp from
                                  {4, 16, 64}, depth 6, seeds 0-63.
  * ``differentiable_scene``    - icosphere level 7 + box (about 200k triangles), per-triangle albedo
                                  U[0.1, 0.9], emission on 64 triangles: the gradient workload.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "icosphere", "displace_value_noise", "box", "quad", "outward_ok", "flat_normals",
    "box_and_icosphere", "displaced_icosphere", "full_scene", "camera_basis", "primary_rays",
    "incoherent_rays", "tri_hash_u32", "random_boxes", "batch_workload", "differentiable_scene",
]


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def icosphere_mesh(level: int):
    """Unit icosphere as (vertices float64 [V,3], faces int64 [F,3]); 20 * 4**level faces,
    counter-clockwise seen from outside."""
    v, f = _icosahedron()
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        key = e[:, 0] * (len(v) + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (len(v) + 1)
        b = uniq % (len(v) + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + len(v)      # midpoints of edges 01, 12, 20
        v = np.concatenate([v, mid], axis=0)
        f0, f1, f2 = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([
            np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
            np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f


def _to_dumbray_winding(tris: np.ndarray) -> np.ndarray:
    """CCW-from-outside triangles -> DumbRay winding (swap b and c)."""
    return tris[:, [0, 2, 1], :]


def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    v, f = icosphere_mesh(level)
    tris = v[f] * radius + np.asarray(center, dtype=np.float64)
    return _to_dumbray_winding(tris).astype(np.float32)


def _value_noise(p: np.ndarray, seed: int, period: int = 256) -> np.ndarray:
    """Trilinear value noise with smoothstep fade over a seeded random lattice (values in [0,1])."""
    rng = np.random.default_rng(seed)
    lat = rng.random(period ** 3)
    i = np.floor(p).astype(np.int64)
    f = p - i
    w = f * f * (3.0 - 2.0 * f)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                idx = (((i[:, 0] + dx) % period) * period + ((i[:, 1] + dy) % period)) * period + ((i[:, 2] + dz) % period)
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += lat[idx] * wx * wy * wz
    return out


def displace_value_noise(v: np.ndarray, amplitude: float, seed: int, octaves: int = 3, base_freq: float = 4.0) -> np.ndarray:
    """Radial displacement of unit-sphere vertices by fractal value noise in [-amplitude, amplitude]."""
    total = np.zeros(len(v))
    norm = 0.0
    for k in range(octaves):
        a = 0.5 ** k
        total += a * (2.0 * _value_noise(v * (base_freq * 2 ** k) + 17.0 * (k + 1), seed + 7919 * k) - 1.0)
        norm += a
    return v * (1.0 + amplitude * total / norm)[:, None]


def displaced_icosphere(level: int = 8, amplitude: float = 0.1, seed: int = 1, radius: float = 1.0,
                        center=(0.0, 0.0, 0.0)) -> np.ndarray:
    v, f = icosphere_mesh(level)
    v = displace_value_noise(v, amplitude, seed) * radius + np.asarray(center, dtype=np.float64)
    return _to_dumbray_winding(v[f]).astype(np.float32)


def box(size=(2.0, 2.0, 2.0), center=(0.0, 0.0, 0.0), inward: bool = False) -> np.ndarray:
    """12-triangle axis-aligned box. Faces in order -x,+x,-y,+y,-z,+z (two triangles each).
    ``inward`` flips the winding so normals face the inside (a room seen from within)."""
    sx, sy, sz = (s * 0.5 for s in size)
    c = np.asarray(center, dtype=np.float64)
    out = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            n = np.zeros(3); n[axis] = sign
            u = np.zeros(3); u[(axis + 1) % 3] = 1.0
            w = np.cross(n, u)
            half = np.array([sx, sy, sz])
            ctr = n * half[axis]
            hu = u * half[(axis + 1) % 3]
            hw = w * half[(axis + 2) % 3]
            p0, p1, p2, p3 = ctr - hu - hw, ctr + hu - hw, ctr + hu + hw, ctr - hu + hw
            # CCW seen from +n
            out.append([p0, p1, p2])
            out.append([p0, p2, p3])
    tris = np.asarray(out) + c
    tris = _to_dumbray_winding(tris)
    if inward:
        tris = tris[:, [0, 2, 1], :]
    return tris.astype(np.float32)


def quad(center, size, normal, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """Two triangles of a size[0] x size[1] rectangle whose DumbRay outward normal is ``normal``."""
    n = np.asarray(normal, dtype=np.float64); n /= np.linalg.norm(n)
    u = np.cross(np.asarray(up, dtype=np.float64), n)
    if np.linalg.norm(u) < 1e-6:
        u = np.cross(np.array([1.0, 0.0, 0.0]), n)
    u /= np.linalg.norm(u)
    w = np.cross(n, u)
    c = np.asarray(center, dtype=np.float64)
    hu, hw = u * size[0] * 0.5, w * size[1] * 0.5
    p0, p1, p2, p3 = c - hu - hw, c + hu - hw, c + hu + hw, c - hu + hw
    tris = np.asarray([[p0, p1, p2], [p0, p2, p3]])
    return _to_dumbray_winding(tris).astype(np.float32)


def dumbray_normal(tris: np.ndarray) -> np.ndarray:
    """Triangle::normal() = (c - a) x (b - a), unnormalised."""
    t = tris.astype(np.float64)
    return np.cross(t[:, 2] - t[:, 0], t[:, 1] - t[:, 0])


def outward_ok(tris: np.ndarray, inside_point) -> np.ndarray:
    """True where the DumbRay normal points away from ``inside_point``."""
    n = dumbray_normal(tris)
    ctr = tris.astype(np.float64).mean(axis=1)
    return (np.einsum("ij,ij->i", n, ctr - np.asarray(inside_point)) > 0)


def flat_normals(tris: np.ndarray) -> np.ndarray:
    n = dumbray_normal(tris)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return np.repeat(n[:, None, :], 3, axis=1).astype(np.float32)


def tri_hash_u32(i: np.ndarray, seed: int = 0) -> np.ndarray:
    """lowbias32 integer hash of the triangle index (used to assign materials)."""
    x = (np.asarray(i, dtype=np.uint64) ^ np.uint64(seed * 0x9E3779B9 & 0xFFFFFFFF)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(16); x = (x * np.uint64(0x7feb352d)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(15); x = (x * np.uint64(0x846ca68b)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(16)
    return x.astype(np.uint32)


def box_and_icosphere(level: int = 5):
    """Plain path-trace scene: 2x2x2 room (inward walls, albedo 0.7, the -x wall red 0.7/0.1/0.1),
    icosphere level ``level`` (r 0.6, centre), one 0.5x0.5 emissive quad (radiance 10) just below
    the ceiling facing down.  Returns dict(tris, mat_id, kind) with materials
    0 = white Lambert, 1 = red Lambert, 2 = emitter."""
    room = box((2.0, 2.0, 2.0), inward=True)
    sphere = icosphere(level, radius=0.6)
    light = quad((0.0, 0.999, 0.0), (0.5, 0.5), (0.0, -1.0, 0.0))
    tris = np.concatenate([room, sphere, light], axis=0)
    mat = np.zeros(len(tris), dtype=np.int32)
    mat[0:2] = 1                      # -x wall red
    mat[len(room) + len(sphere):] = 2
    return dict(tris=tris, mat_id=mat, n_room=len(room), n_sphere=len(sphere), n_light=len(light))


def full_scene(level: int = 8, seed: int = 1):
    """Displaced icosphere (r 1) standing on a ground plane, lit by 4 emissive quads.
    Materials by triangle-index hash: <60 Lambert (albedo U[0.2,0.8]^3), <85 mirror, else glossy
    (roughness U[0.05,0.4]).  Returns dict(tris, mat_id, albedo, roughness, emission)."""
    mesh = displaced_icosphere(level, 0.1, seed)
    ground = quad((0.0, -1.2, 0.0), (40.0, 40.0), (0.0, 1.0, 0.0))
    lights = np.concatenate([
        quad((x, 3.0, z), (1.0, 1.0), (0.0, -1.0, 0.0)) for x, z in ((-2.0, -2.0), (2.0, -2.0), (-2.0, 2.0), (2.0, 2.0))
    ], axis=0)
    tris = np.concatenate([mesh, ground, lights], axis=0)
    n = len(tris)
    h = tri_hash_u32(np.arange(n), seed) % 100
    mat = np.where(h < 60, 0, np.where(h < 85, 1, 2)).astype(np.int32)
    rng = np.random.default_rng(seed)
    albedo = rng.uniform(0.2, 0.8, size=(n, 3)).astype(np.float32)
    rough = rng.uniform(0.05, 0.4, size=n).astype(np.float32)
    nm = len(mesh)
    mat[nm:nm + len(ground)] = 0
    albedo[nm:nm + len(ground)] = 0.5
    mat[nm + len(ground):] = 0
    emission = np.zeros((n, 3), dtype=np.float32)
    emission[nm + len(ground):] = 10.0
    albedo[nm + len(ground):] = 0.0
    return dict(tris=tris, mat_id=mat, albedo=albedo, roughness=rough, emission=emission,
                n_mesh=nm, n_ground=len(ground), n_lights=len(lights))


def camera_basis(position, target, up=(0.0, 1.0, 0.0)):
    p = np.asarray(position, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - p
    f /= np.linalg.norm(f)
    r = np.cross(np.asarray(up, dtype=np.float64), f)
    r /= np.linalg.norm(r)
    u = np.cross(f, r)
    return p.astype(np.float32), r.astype(np.float32), u.astype(np.float32), f.astype(np.float32)


def primary_rays(width: int, height: int, fov_deg: float, position, target):
    """Coherent pinhole camera rays through pixel centres, normalised directions (row-major)."""
    p, r, u, f = camera_basis(position, target)
    x = 0.5 / np.tan(np.radians(fov_deg) / 2.0)
    ps = 1.0 / height
    xs = (np.arange(width) + 0.5 - width / 2.0) * ps
    ys = (height / 2.0 - (np.arange(height) + 0.5)) * ps
    sx, sy = np.meshgrid(xs, ys)
    d = sx[..., None] * r + sy[..., None] * u + x * f
    d = d.reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(p, d.shape)
    return np.ascontiguousarray(o, dtype=np.float32), np.ascontiguousarray(d, dtype=np.float32)


def incoherent_rays(n: int, lo, hi, seed: int = 0):
    """Origins uniform in the box [lo, hi], directions uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def random_boxes(n: int, rng, lo=-1.6, hi=1.6, fill=0.25) -> np.ndarray:
    """``n`` closed axis-aligned boxes (12 triangles each, outward normals), centres uniform in
    [lo, hi]^3, edge lengths uniform in [0.5 e, 1.5 e] with e chosen so that the boxes' summed
    volume is ``fill`` of the region's (the box density stays the same whatever ``n`` is)."""
    if n <= 0:
        return np.zeros((0, 3, 3), np.float32)
    unit = box((1.0, 1.0, 1.0)).astype(np.float64)              # [12, 3, 3]
    e = (fill * (hi - lo) ** 3 / n) ** (1.0 / 3.0)
    ext = rng.uniform(0.5 * e, 1.5 * e, size=(n, 1, 1, 3))
    ctr = rng.uniform(lo, hi, size=(n, 1, 1, 3))
    return (unit[None] * ext + ctr).reshape(-1, 3, 3).astype(np.float32)


_DISPLACED_CACHE: dict = {}


def _displaced_level(level: int) -> np.ndarray:
    if level not in _DISPLACED_CACHE:
        _DISPLACED_CACHE[level] = displaced_icosphere(level, 0.1, 1)
    return _DISPLACED_CACHE[level]


def _rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def batch_workload(n_scenes: int = 64, seed: int = 0, min_tris: int = 1000, max_tris: int = 2_000_000,
                   resolutions=(128, 256, 512, 1024), spps=(4, 16, 64), depth: int = 6):
    """The batched-rendering workload: ``n_scenes`` independent scenes.

    Scene i: target triangle count T log-uniform in [min_tris, max_tris]; the largest displaced
    icosphere (3-octave value noise, amplitude 0.1) with at most T triangles, randomly rotated and
    scaled to radius U[0.5, 0.9], plus ceil((T - icosphere) / 12) random boxes around it (summed box
    volume a quarter of the [-1.6, 1.6]^3 region, whatever their number), a 2-triangle
    ground plane and one emissive quad (radiance 10) above; materials by triangle-index hash as in
    ``full_scene``.  Resolution square, uniform from ``resolutions``; spp uniform from ``spps``;
    render seed i.  Returns a list of dicts (tris, mat_id, albedo, roughness, emission, width,
    height, spp, depth, seed, camera position/target)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        target = int(round(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris)))))
        level = 0
        while 20 * 4 ** (level + 1) <= target and level < 8:
            level += 1
        mesh = _displaced_level(level).astype(np.float64)
        rot = _rotation(rng)
        radius = rng.uniform(0.5, 0.9)
        mesh = (mesh @ rot.T * radius).astype(np.float32)
        n_boxes = max(0, -(-(target - len(mesh)) // 12))
        boxes = random_boxes(n_boxes, rng)
        ground = quad((0.0, -1.7, 0.0), (12.0, 12.0), (0.0, 1.0, 0.0))
        light = quad((0.0, 2.5, 0.0), (1.5, 1.5), (0.0, -1.0, 0.0))
        tris = np.concatenate([mesh, boxes, ground, light], axis=0)
        n = len(tris)
        h = tri_hash_u32(np.arange(n), i) % 100
        mat = np.where(h < 60, 0, np.where(h < 85, 1, 2)).astype(np.int32)
        albedo = rng.uniform(0.2, 0.8, size=(n, 3)).astype(np.float32)
        rough = rng.uniform(0.05, 0.4, size=n).astype(np.float32)
        mat[-4:] = 0
        albedo[-4:-2] = 0.5
        albedo[-2:] = 0.0
        emission = np.zeros((n, 3), np.float32)
        emission[-2:] = 10.0
        res = int(rng.choice(resolutions))
        spp = int(rng.choice(spps))
        ang = rng.uniform(0.0, 2.0 * np.pi)
        cam_pos = (float(3.4 * np.sin(ang)), 0.8, float(-3.4 * np.cos(ang)))
        out.append(dict(tris=tris, mat_id=mat, albedo=albedo, roughness=rough, emission=emission, width=res,
                        height=res, spp=spp, depth=depth, seed=i, cam_pos=cam_pos, cam_target=(0.0, 0.0, 0.0),
                        target_tris=target, level=level, n_boxes=n_boxes))
    return out


def differentiable_scene(level: int = 7, n_emissive: int = 64, seed: int = 7):
    """Gradient workload: icosphere ``level`` (327,680 triangles at level 7 is the next subdivision
    above 200k; level 7 it is) of radius 0.6 inside a 12-triangle 2x2x2 room; per-triangle albedo
    U[0.1, 0.9]^3 (Lambert); emission 10 on ``n_emissive`` sphere triangles picked by a seeded hash.
    Returns dict(tris, mat_id, albedo, emission, roughness, emissive_ids) and hidden target
    parameters (albedo_target = an independent U[0.1, 0.9] draw, same emission)."""
    room = box((2.0, 2.0, 2.0), inward=True)
    sphere = icosphere(level, radius=0.6)
    tris = np.concatenate([room, sphere], axis=0)
    n = len(tris)
    rng = np.random.default_rng(seed)
    albedo = rng.uniform(0.1, 0.9, size=(n, 3)).astype(np.float32)
    albedo_target = rng.uniform(0.1, 0.9, size=(n, 3)).astype(np.float32)
    ids = len(room) + np.sort(rng.choice(len(sphere), size=n_emissive, replace=False))
    emission = np.zeros((n, 3), np.float32)
    emission[ids] = 10.0
    return dict(tris=tris, mat_id=np.zeros(n, np.int32), albedo=albedo, albedo_target=albedo_target,
                emission=emission, roughness=np.full(n, 0.2, np.float32), emissive_ids=ids, n_room=len(room))
