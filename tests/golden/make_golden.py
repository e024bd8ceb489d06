"""Generates the golden fixtures in tests/golden/ by running the REFERENCE DumbRay host path
(oracle/_ref/libdumbref.so, compiled from the reference sources by oracle/build_ref.sh).

  cast_small.npz   displaced icosphere level 4 + inward 3x3x3 box (5,132 tris); 8,192 incoherent rays
                   and 64x48 pinhole primaries; reference Octree::cast hit index and t, culling on and
                   off; reference node count.
  cast_c1.npz      the 20,492-triangle box + icosphere level 5 geometry; 16,384 incoherent rays,
                   culling on.
  cast_c2_l8.npz   the ray-cast microbenchmark mesh itself (icosphere level 8, 1,310,720 triangles,
                   radially displaced by 3-octave value noise, amplitude 0.1, seed 1; stored as its
                   SHA-256, regenerated by the tests): 8,192 of the benchmark's incoherent rays (origins
                   uniform in [-1.1, 1.1]^3, seed 0) and 8,100 of its 1920x1080 pinhole primaries (every
                   256th); reference Octree::cast index and t, culling on and off; reference node count.
  render_c3_twin.npz  the reference-expressible twin of the full path-trace scene (bench.reference_twin:
                   the level-8 displaced icosphere on a ground plane, DumbBased diffuse / metal and
                   SimpleStochastic mirror materials by triangle hash, 4 spherical lights; the
                   SimpleStochasticLense 60-degree view of the benchmark frame at 96x54, depth 8): four
                   reference DumbRenderer runs of 256 iterations, float16 RGB.
  render_c1_twin.npz  the reference-expressible twin of the 256x256 box + icosphere scene (c1_twin):
                   four reference DumbRenderer runs of 64 iterations at 256x256, depth 4, stored as
                   float16 RGB (quantisation far below the Monte Carlo noise).
  render_*.npz     reference DumbRenderer CPU renders (four independent runs of 512 progressive
                   iterations each) of small reference-expressible scenes, 32x32: a room and a sphere
                   of each reference shader (DumbBased diffuse / metal, SimpleStochastic, Fresnel,
                   Default) under a spherical light, and under spotlights (disc emitter with shadows;
                   sphere emitter without shadows beside a soft directional light).
  render_tex_*.npz the same reference renders of textured scenes (texture_scene: textured diffuse
                   and fresnel channels with tiling / offset, a normal map, an alpha-cutout screen,
                   a textured Fresnel shader; nearest and bilinear filtering), 32x32.
  scene_file/      a scene file (scene.dumb including materials.dumb, meshes in props.obj) that uses
                   presets, groups with fallback / override materials, rotated and scaled items and a
                   rotated spherical-segment camera; render_scene_file.npz holds the reference's renders
                   of it, loaded by the reference's own DumbRenderContext::fromFile (four runs of 512
                   iterations, 32x24).
  scene_file_tex/  a textured scene file (PNG textures by path and by name, nearest / bilinear, tiling
                   and offsets, a normal map, an alpha-cutout screen, a textured fresnel_color; an OBJ
                   with texture coordinates); render_scene_file_tex.npz as above, 32x32.

Run from the repository root after `bash oracle/build_ref.sh`:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import dumbray_gb300 as dr  # noqa: E402
from dumbray_gb300 import scenes  # noqa: E402
import _oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def cast_fixtures():
    tris = np.concatenate([scenes.displaced_icosphere(4, 0.1, 1), scenes.box((3.0, 3.0, 3.0), inward=True)])
    oi, di = scenes.incoherent_rays(8192, -1.2, 1.2, seed=5)
    op, dp = scenes.primary_rays(64, 48, 60.0, (0.3, 0.4, -3.0), (0.0, 0.0, 0.0))
    o = np.concatenate([oi, op])
    d = np.concatenate([di, dp])
    out = dict(tris=tris, o=o, d=d)
    for cull in (1, 0):
        idx, t, nodes = O.ref_cast(tris, o, d, cull=bool(cull))
        out[f"idx_cull{cull}"] = idx
        out[f"t_cull{cull}"] = t
        out["nodes"] = np.int64(nodes)
    np.savez_compressed(OUT / "cast_small.npz", **out)

    c1 = scenes.box_and_icosphere(5)
    tris = c1["tris"]
    o, d = scenes.incoherent_rays(16384, -0.95, 0.95, seed=9)
    idx, t, nodes = O.ref_cast(tris, o, d, cull=True)
    np.savez_compressed(OUT / "cast_c1.npz", tris=tris, o=o, d=d, idx_cull1=idx, t_cull1=t, nodes=np.int64(nodes))


def mesh_sha256(tris) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(tris, np.float32).tobytes()).hexdigest()


def c2_rays():
    """The C2 subset: the first 8,192 of 8,192 incoherent rays drawn like the benchmark's (seed 0)
    and every 256th of the 1920x1080 primaries (60 degrees from (0, 0.3, -3) toward the origin)."""
    oi, di = scenes.incoherent_rays(8192, -1.1, 1.1, seed=0)
    op, dp = scenes.primary_rays(1920, 1080, 60.0, (0.0, 0.3, -3.0), (0.0, 0.0, 0.0))
    return np.concatenate([oi, op[::256]]), np.concatenate([di, dp[::256]])


def cast_c2_fixture():
    tris = scenes.displaced_icosphere(8, 0.1, 1)
    o, d = c2_rays()
    out = dict(o=o, d=d, mesh_sha256=np.array(mesh_sha256(tris)), n_tris=np.int64(len(tris)))
    for cull in (1, 0):
        idx, t, nodes = O.ref_cast(tris, o, d, cull=bool(cull))
        out[f"idx_cull{cull}"] = idx
        out[f"t_cull{cull}"] = t
        out["nodes"] = np.int64(nodes)
    np.savez_compressed(OUT / "cast_c2_l8.npz", **out)
    print("cast_c2_l8: nodes", int(out["nodes"]), "hit fraction", float((out["idx_cull1"] >= 0).mean()))


C1_SIZE, C1_DEPTH = 256, 4


def c1_twin():
    """Reference-expressible twin of the plain path-trace scene (2x2x2 room, icosphere level 5 of
    radius 0.6, 0.5x0.5 emissive quad of radiance 10 below the ceiling): the room and the sphere keep
    their geometry with DumbBasedShader diffuse (metal 0) albedo 0.7 and the red wall 0.7/0.1/0.1;
    the quad becomes a SphericalLightEmitter of the same power (radiance x area x pi over 4 pi per
    channel, radius 0.05).  The emitter sits at y = 0.8, midway between the sphere's top (0.6) and
    the ceiling (1.0), instead of on the ceiling: a point emitter touching a wall makes the
    reference's 1/d^2 photons heavy-tailed, and four reference runs cannot then estimate the
    standard error.  Lens: SimpleStochasticLense 60 degrees from (0, 0, -0.99).
    Returns (tris, mat, mats, lights, cam)."""
    c = scenes.box_and_icosphere(5)
    n_geo = c["n_room"] + c["n_sphere"]
    tris, mat = c["tris"][:n_geo], c["mat_id"][:n_geo].copy()
    mats = [dr.dumb_based(diffuse=(0.7, 0.7, 0.7), metal=0.0), dr.dumb_based(diffuse=(0.7, 0.1, 0.1), metal=0.0)]
    power = 10.0 * 0.25 * np.pi
    lights = [dr.spherical_light((power / (4.0 * np.pi),) * 3, (0.0, 0.8, 0.0), 0.05)]
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.99), angle=60.0)
    return tris, mat, mats, lights, cam


def render_c1_twin_fixture(iterations=64, runs=4):
    tris, mat, mats, lights, cam = c1_twin()
    out, secs = [], 0.0
    for _ in range(runs):
        img, t = O.ref_render(tris, mat, mats, lights, cam, C1_SIZE, C1_SIZE, max_bounces=C1_DEPTH,
                              iterations=iterations)
        out.append(img[..., :3].astype(np.float16))
        secs += t
    runs_arr = np.stack(out)
    np.savez_compressed(OUT / "render_c1_twin.npz", runs=runs_arr, iterations=np.int64(iterations),
                        size=np.int64(C1_SIZE), bounces=np.int64(C1_DEPTH), seconds=np.float64(secs))
    print("c1 twin: reference seconds", secs, "mean", runs_arr.astype(np.float64).mean())


C3_W, C3_H, C3_DEPTH = 96, 54, 8


def c3_twin():
    """(tris, mat, mats, lights, cam) of the full path-trace scene's reference-expressible twin, as the
    benchmark's reference-mode leg and reference arm render it."""
    import bench
    S = scenes.full_scene(level=8, seed=1)
    tris, mat, mats, lights = bench.reference_twin(S, dr)
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.6, -3.4), angle=60.0)
    return tris, mat, mats, lights, cam


def render_c3_twin_fixture(iterations=256, runs=4):
    tris, mat, mats, lights, cam = c3_twin()
    out, secs = [], 0.0
    for _ in range(runs):
        img, t = O.ref_render(tris, mat, mats, lights, cam, C3_W, C3_H, max_bounces=C3_DEPTH, iterations=iterations)
        out.append(img[..., :3].astype(np.float16))
        secs += t
    runs_arr = np.stack(out)
    np.savez_compressed(OUT / "render_c3_twin.npz", runs=runs_arr, iterations=np.int64(iterations),
                        width=np.int64(C3_W), height=np.int64(C3_H), bounces=np.int64(C3_DEPTH),
                        seconds=np.float64(secs))
    print("c3 twin: reference seconds", secs, "mean", runs_arr.astype(np.float64).mean())


def render_scene(kind: str):
    room = scenes.box((2.0, 2.0, 2.0), inward=True)
    sph = scenes.icosphere(2, 0.5)
    tris = np.concatenate([room, sph])
    mat = np.zeros(len(tris), np.int32)
    mat[0:2] = 1
    mat[len(room):] = 2
    white = dr.dumb_based(diffuse=(0.7, 0.7, 0.7), metal=0.0)
    red = dr.dumb_based(diffuse=(0.7, 0.1, 0.1), metal=0.0)
    if kind in ("diffuse", "spot", "spot_open"):
        obj = dr.dumb_based(diffuse=(0.5, 0.6, 0.7), metal=0.0)
    elif kind == "metal":
        obj = dr.dumb_based(fresnel=(1.022, 0.782, 0.344), specular=16.0, diffuse=(1.0, 1.0, 1.0), metal=0.5)
    elif kind == "fresnel":
        obj = dr.fresnel_shader((0.9, 0.6, 0.3))
    elif kind == "default":
        obj = dr.default_shader((0.8, 0.8, 0.9), 0.5, 0.4, 16.0)
    else:
        obj = dr.simple_stochastic((0.9, 0.9, 0.9), 0.3, 0.7, 8.0)
    mats = [white, red, obj]
    if kind == "spot":
        lights = [dr.spotlight((1.0, 0.95, 0.9), 150.0, (0.0, 0.9, 0.0), (0.1, -1.0, 0.15), 20.0, 50.0, 1.5, 0.1,
                               emit_from_sphere=False, cast_shadows=True, samples=4)]
    elif kind == "spot_open":
        # emitter and shadowed light kept away from every surface (no near-singular 1/d^2 samples)
        lights = [dr.spotlight((0.9, 0.95, 1.0), 60.0, (0.3, 0.75, -0.2), (-0.2, -1.0, 0.1), 25.0, 60.0, 1.0, 0.08,
                               emit_from_sphere=True, cast_shadows=False, samples=3),
                  dr.soft_directional_light((0.3, 0.3, 0.3), (0.3, -1.0, 0.2), 3.0, 0.05)]
    else:
        lights = [dr.spherical_light((1.5, 1.5, 1.5), (0.0, 0.8, 0.0), 0.1)]
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.95), angle=60.0)
    return tris, mat, mats, lights, cam


RENDER_KINDS = ("diffuse", "metal", "ss", "fresnel", "default", "spot", "spot_open")


def render_fixtures(iterations=512, runs=4, size=32, bounces=2, kinds=RENDER_KINDS):
    for kind in kinds:
        tris, mat, mats, lights, cam = render_scene(kind)
        out, secs = [], 0.0
        for _ in range(runs):
            img, t = O.ref_render(tris, mat, mats, lights, cam, size, size, max_bounces=bounces, iterations=iterations)
            out.append(img)
            secs += t
        runs_arr = np.stack(out)
        np.savez_compressed(OUT / f"render_{kind}.npz", runs=runs_arr, iterations=np.int64(iterations),
                            size=np.int64(size), bounces=np.int64(bounces), seconds=np.float64(secs))
        print(kind, "reference seconds", secs, "mean", runs_arr[..., :3].mean())


def _room_uv(room):
    """Planar texture coordinates of the room's walls: the two coordinates along each face."""
    uv = np.zeros((len(room), 3, 2), np.float32)
    for i, t in enumerate(room):
        n = np.abs(np.cross(t[1] - t[0], t[2] - t[0]))
        ax = int(np.argmax(n))
        a, b = [k for k in range(3) if k != ax]
        uv[i, :, 0] = t[:, a] * 0.5 + 0.5
        uv[i, :, 1] = t[:, b] * 0.5 + 0.5
    return uv


def _sphere_uv(sph):
    """Spherical texture coordinates of the sphere's corners."""
    p = sph.astype(np.float64)
    r = np.linalg.norm(p, axis=-1)
    u = 0.5 + np.arctan2(p[..., 2], p[..., 0]) / (2 * np.pi)
    v = 0.5 + np.arcsin(np.clip(p[..., 1] / r, -1, 1)) / np.pi
    return np.stack([u, v], axis=-1).astype(np.float32)


def _texture(kind, size, seed):
    rng = np.random.default_rng(seed)
    h, w = size
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.ones((h, w, 4), np.float32)
    if kind == "checker":
        c = ((xx // 2 + yy // 2) % 2).astype(np.float32)
        img[..., :3] = 0.25 + 0.6 * c[..., None] * np.array([1.0, 0.8, 0.6], np.float32)
    elif kind == "noise":
        img[..., :3] = rng.uniform(0.2, 1.0, size=(h, w, 3)).astype(np.float32)
    elif kind == "bumps":
        a = 2 * np.pi * xx / w
        b = 2 * np.pi * yy / h
        img[..., 0] = 0.5 + 0.25 * np.sin(a * 2)
        img[..., 1] = 0.5 + 0.25 * np.cos(b * 3)
        img[..., 2] = 0.9
    elif kind == "stripes":
        img[..., :3] = 0.8
        img[..., 3] = ((xx // 3) % 2).astype(np.float32)
    return img


def texture_scene(kind: str):
    """Textured scenes: the render_scene room and sphere with texture coordinates (planar on the walls,
    spherical on the sphere) and textures from _texture.  Returns (tris, mat, mats, lights, cam, uv,
    textures); textures are [(rgba, filtering)]."""
    room = scenes.box((2.0, 2.0, 2.0), inward=True)
    sph = scenes.icosphere(2, 0.5)
    parts = [room, sph]
    uvs = [_room_uv(room), _sphere_uv(sph)]
    white = dr.dumb_based(diffuse=(0.7, 0.7, 0.7), metal=0.0)
    red = dr.dumb_based(diffuse=(0.7, 0.1, 0.1), metal=0.0)
    textures = [(_texture("checker", (16, 16), 1), dr.FILTER_BILINEAR), (_texture("noise", (8, 8), 2), dr.FILTER_NONE),
                (_texture("bumps", (32, 32), 3), dr.FILTER_BILINEAR), (_texture("stripes", (12, 12), 4), dr.FILTER_NONE)]
    if kind == "tex_diffuse":
        obj = dr.textured(dr.textured(dr.dumb_based(fresnel=(0.6, 0.5, 0.4), specular=32.0, diffuse=(0.9, 0.9, 0.9), metal=0.3),
                                      dr.TEX_COLOR, 0, (2.0, 1.5), (0.1, -0.2)), dr.TEX_FRESNEL, 1)
        white = dr.textured(white, dr.TEX_COLOR, 1, (3.0, 3.0))
    elif kind == "tex_normal":
        obj = dr.textured(dr.textured(dr.dumb_based(fresnel=(0.9, 0.8, 0.6), specular=24.0, diffuse=(0.8, 0.7, 0.6), metal=0.6),
                                      dr.TEX_NORMAL, 2, (2.0, 2.0)), dr.TEX_COLOR, 0)
        obj.normal_color[:] = (1.0, 0.8, 0.9)
    elif kind == "tex_alpha":
        obj = dr.dumb_based(diffuse=(0.5, 0.6, 0.7), metal=0.0)
        screen = scenes.quad((0.0, 0.0, -0.6), (1.2, 1.2), (0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0))
        parts.append(screen)
        uvs.append(np.array([[[x * 0.5 + 0.5, y * 0.5 + 0.5] for x, y, _ in t] for t in screen / 0.6], np.float32))
    else:  # tex_fresnel
        obj = dr.textured(dr.fresnel_shader((0.9, 0.6, 0.3)), dr.TEX_COLOR, 0, (4.0, 2.0))
    tris = np.concatenate(parts)
    uv = np.concatenate(uvs)
    mat = np.zeros(len(tris), np.int32)
    mat[0:2] = 1
    mat[len(room):len(room) + len(sph)] = 2
    mats = [white, red, obj]
    if kind == "tex_alpha":
        mat[len(room) + len(sph):] = 3
        mats.append(dr.textured(dr.dumb_based(diffuse=(0.9, 0.4, 0.2), metal=0.0), dr.TEX_ALPHA, 3, (1.0, 1.0)))
    lights = [dr.spherical_light((1.5, 1.5, 1.5), (0.0, 0.8, 0.0), 0.1)]
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.95), angle=60.0)
    return tris, mat, mats, lights, cam, uv, textures


TEXTURE_KINDS = ("tex_diffuse", "tex_normal", "tex_alpha", "tex_fresnel")


def texture_fixtures(iterations=512, runs=4, size=32, bounces=2, kinds=TEXTURE_KINDS):
    for kind in kinds:
        tris, mat, mats, lights, cam, uv, textures = texture_scene(kind)
        out, secs = [], 0.0
        for _ in range(runs):
            img, t = O.ref_render(tris, mat, mats, lights, cam, size, size, max_bounces=bounces, iterations=iterations,
                                  uv=uv, textures=textures)
            out.append(img)
            secs += t
        runs_arr = np.stack(out)
        np.savez_compressed(OUT / f"render_{kind}.npz", runs=runs_arr, iterations=np.int64(iterations),
                            size=np.int64(size), bounces=np.int64(bounces), seconds=np.float64(secs))
        print(kind, "reference seconds", secs, "mean", runs_arr[..., :3].mean())


SCENE_FILE_DIR = OUT / "scene_file"

SCENE_FILE_MATERIALS = """{
	"materials": [
		{ "name": "walls", "type": "dumb_based", "preset": "matte", "diffuse": [ 0.7, 0.7, 0.7 ] },
		{ "name": "red", "type": "dumb_based", "preset": "matte", "diffuse": [ 0.7, 0.1, 0.1 ], "fresnel": [ 0.3, 0.2, 0.2 ] },
		{ "name": "gold", "type": "dumb_based", "preset": "gold", "specular": 24 },
		{ "name": "chalk", "type": "simple_stochastic", "color": [ 0.9, 0.85, 0.8 ], "diffuse": 0.3, "smoothness": 0.6, "shininess": 8 }
	]
}
"""

SCENE_FILE_MAIN = """{
	"include": [ "materials.dumb" ],
	"lights": [
		{ "type": "simple_spherical", "color": [ 1.5, 1.5, 1.4 ], "position": [ 0, 0.8, 0 ], "radius": 0.1 },
		{ "type": "simple_soft_directional", "color": [ 0.1, 0.1, 0.12 ] }
	],
	"groups": [
		{
			"name": "props",
			"elements": [
				{ "mesh": { "obj": "props.obj", "object": "sphere" },
				  "transform": { "position": [ 0.3, -0.5, 0.25 ], "scale": [ 0.6, 0.6, 0.6 ] },
				  "material": "gold" },
				{ "mesh": { "obj": "props.obj", "object": "cube" },
				  "transform": { "position": [ -0.4, -0.75, 0.3 ], "rotation": [ 20, 30, 0 ], "scale": [ 0.3, 0.3, 0.3 ] } }
			],
			"fallback_material": "chalk",
			"transform": { "position": [ 0, 0.05, 0 ] }
		}
	],
	"objects": [
		{ "mesh": { "obj": "props.obj", "object": "room" }, "material": "walls" },
		{ "group": "props", "transform": { "rotation": [ 0, 15, 0 ] } },
		{
			"elements": [
				{ "mesh": { "obj": "props.obj", "object": "cube" },
				  "transform": { "position": [ 0.55, -0.8, -0.2 ], "rotation": [ 0, 45, 10 ], "scale": [ 0.25, 0.35, 0.25 ] } }
			],
			"override_material": "red",
			"transform": { "position": [ 0, 0.02, 0 ] }
		}
	],
	"camera": {
		"lense": { "type": "spherical_segment", "angle": 70, "distance": 1.6, "sensor": 0.01, "filter": [ 1, 0.95, 0.9 ] },
		"transform": { "position": [ 0, 0.05, -0.55 ], "rotation": [ 6, -9, 3 ], "relative_position": [ 0, 0, -0.3 ] }
	},
	"renderer": {
		"pixel": { "boxing": "width", "bounces": 2, "samples_per_pixel": [ 1, 1 ] }
	}
}
"""


def _obj_text(objects, uvs=None):
    """OBJ text with one `g` group per (name, triangles); x is written negated because the reader
    mirrors it back.  ``uvs``: optional per-object corner texture coordinates [n, 3, 2] (`vt` lines)."""
    lines, base = [], 1
    for k, (name, tris) in enumerate(objects):
        lines.append(f"g {name}")
        for t in tris:
            for v in t:
                lines.append(f"v {-float(v[0]):.9g} {float(v[1]):.9g} {float(v[2]):.9g}")
        if uvs is not None:
            for t in uvs[k]:
                for c in t:
                    lines.append(f"vt {float(c[0]):.9g} {float(c[1]):.9g}")
        for i in range(len(tris)):
            a, b, c = base + 3 * i, base + 3 * i + 1, base + 3 * i + 2
            lines.append(f"f {a}/{a} {b}/{b} {c}/{c}" if uvs is not None else f"f {a} {b} {c}")
        base += 3 * len(tris)
    return "\n".join(lines) + "\n"


def write_scene_file(directory=SCENE_FILE_DIR):
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    objects = [("room", scenes.box((2.0, 2.0, 2.0), inward=True)), ("sphere", scenes.icosphere(2, 0.5)),
               ("cube", scenes.box((1.0, 1.0, 1.0)))]
    (directory / "props.obj").write_text(_obj_text(objects))
    (directory / "materials.dumb").write_text(SCENE_FILE_MATERIALS)
    (directory / "scene.dumb").write_text(SCENE_FILE_MAIN)
    return directory / "scene.dumb"


SCENE_FILE_TEX_DIR = OUT / "scene_file_tex"

SCENE_FILE_TEX_MAIN = """{
	"materials": [
		{ "name": "walls", "type": "dumb_based", "preset": "matte",
		  "diffuse": [ 0.8, 0.8, 0.8 ], "diffuse_texture": { "png": "checker.png", "name": "checker" }, "diffuse_tiling": [ 3, 3 ] },
		{ "name": "gold", "type": "dumb_based", "preset": "gold", "specular": 24,
		  "fresnel_texture": { "png": "noise.png", "filtering": "none" },
		  "normal_texture": { "png": "bumps.png", "name": "bumps" }, "normal_color": [ 1, 0.8, 0.9 ], "normal_tiling": [ 2, 2 ] },
		{ "name": "painted", "type": "dumb_based", "preset": "glossy", "diffuse": [ 0.9, 0.5, 0.3 ],
		  "diffuse_texture": "checker", "diffuse_offset": [ 0.25, -0.1 ] },
		{ "name": "screen", "type": "dumb_based", "diffuse": [ 0.9, 0.4, 0.2 ], "metal": 0,
		  "alpha_cutout_texture": { "png": "stripes.png", "filtering": "none" }, "alpha_cutout_threshold": 0.4 },
		{ "name": "tinted", "type": "fresnel_color", "engine_color": "copper", "texture": "noise.png", "tiling": [ 4, 2 ] }
	],
	"lights": [ { "type": "simple_spherical", "color": [ 1.5, 1.5, 1.5 ], "position": [ 0, 0.8, 0 ], "radius": 0.1 } ],
	"objects": [
		{ "mesh": { "obj": "textured.obj", "object": "room" }, "material": "walls" },
		{ "mesh": { "obj": "textured.obj", "object": "sphere" }, "material": "gold", "transform": { "position": [ 0.2, -0.4, 0.3 ], "scale": [ 0.7, 0.7, 0.7 ] } },
		{ "mesh": { "obj": "textured.obj", "object": "sphere" }, "material": "tinted", "transform": { "position": [ -0.5, 0.3, 0.4 ], "scale": [ 0.35, 0.35, 0.35 ] } },
		{ "mesh": { "obj": "textured.obj", "object": "cube" }, "material": "painted", "transform": { "position": [ -0.5, -0.8, 0.2 ], "rotation": [ 0, 30, 0 ], "scale": [ 0.35, 0.35, 0.35 ] } },
		{ "mesh": { "obj": "textured.obj", "object": "screen" }, "material": "screen" }
	],
	"camera": { "lense": { "type": "simple_stochastic", "angle": 60 }, "transform": { "position": [ 0, 0, -0.95 ] } },
	"renderer": { "pixel": { "bounces": 2 } }
}
"""


def write_scene_file_textured(directory=SCENE_FILE_TEX_DIR):
    """The textured scene file: textures from _texture written as PNG, an OBJ with texture coordinates."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    room = scenes.box((2.0, 2.0, 2.0), inward=True)
    sph = scenes.icosphere(2, 0.5)
    cube = scenes.box((1.0, 1.0, 1.0))
    screen = scenes.quad((0.0, 0.0, -0.6), (1.2, 1.2), (0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0))
    screen_uv = np.array([[[x * 0.5 + 0.5, y * 0.5 + 0.5] for x, y, _ in t] for t in screen / 0.6], np.float32)
    objects = [("room", room), ("sphere", sph), ("cube", cube), ("screen", screen)]
    uvs = [_room_uv(room), _sphere_uv(sph), _room_uv(cube * 2.0), screen_uv]
    (directory / "textured.obj").write_text(_obj_text(objects, uvs))
    for name, kind, size, seed in (("checker", "checker", (16, 16), 1), ("noise", "noise", (8, 8), 2),
                                   ("bumps", "bumps", (32, 32), 3), ("stripes", "stripes", (12, 12), 4)):
        dr.write_png(_texture(kind, size, seed), directory / f"{name}.png")
    (directory / "scene.dumb").write_text(SCENE_FILE_TEX_MAIN)
    return directory / "scene.dumb"


def scene_file_fixtures(iterations=512, runs=4, width=32, height=24):
    path = write_scene_file()
    out, secs = [], 0.0
    for _ in range(runs):
        img, t = O.ref_dumb_render(path, width, height, iterations)
        out.append(img)
        secs += t
    runs_arr = np.stack(out)
    np.savez_compressed(OUT / "render_scene_file.npz", runs=runs_arr, iterations=np.int64(iterations),
                        width=np.int64(width), height=np.int64(height), seconds=np.float64(secs))
    print("scene file: reference seconds", secs, "mean", runs_arr[..., :3].mean())


def scene_file_tex_fixtures(iterations=512, runs=4, width=32, height=32):
    path = write_scene_file_textured()
    out, secs = [], 0.0
    for _ in range(runs):
        img, t = O.ref_dumb_render(path, width, height, iterations)
        out.append(img)
        secs += t
    runs_arr = np.stack(out)
    np.savez_compressed(OUT / "render_scene_file_tex.npz", runs=runs_arr, iterations=np.int64(iterations),
                        width=np.int64(width), height=np.int64(height), seconds=np.float64(secs))
    print("textured scene file: reference seconds", secs, "mean", runs_arr[..., :3].mean())


if __name__ == "__main__":
    if not O.reference_available():
        raise SystemExit("build the reference first: bash oracle/build_ref.sh")
    only = sys.argv[1:]
    if not only or "cast" in only:
        cast_fixtures()
    if not only or "cast_c2" in only:
        cast_c2_fixture()
    if not only or "render_c1_twin" in only:
        render_c1_twin_fixture()
    if not only or "render_c3_twin" in only:
        render_c3_twin_fixture()
    if not only or "render" in only:
        render_fixtures()
    if not only or "textures" in only:
        texture_fixtures()
    for k in only:
        if k in ("render_c1_twin", "render_c3_twin"):
            continue
        if k.startswith("render_tex_"):
            texture_fixtures(kinds=(k[len("render_"):],))
        elif k.startswith("render_"):
            render_fixtures(kinds=(k[len("render_"):],))
    if not only or "scene_file" in only:
        scene_file_fixtures()
    if not only or "scene_file_tex" in only:
        scene_file_tex_fixtures()
    print("golden fixtures written to", OUT)
