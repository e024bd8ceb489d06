"""Generates the golden fixtures in tests/golden/ by running the REFERENCE DumbRay host path
(oracle/_ref/libdumbref.so, compiled from the reference sources by oracle/build_ref.sh).

  cast_small.npz   displaced icosphere level 4 + inward 3x3x3 box (5,132 tris); 8,192 incoherent rays
                   and 64x48 pinhole primaries; reference Octree::cast hit index and t, culling on and
                   off; reference node count.
  cast_c1.npz      the 20,492-triangle box + icosphere level 5 geometry; 16,384 incoherent rays,
                   culling on.
  render_*.npz     reference DumbRenderer CPU renders (four independent runs of 512 progressive
                   iterations each) of small reference-expressible scenes, 32x32: a room and a sphere
                   of each reference shader (DumbBased diffuse / metal, SimpleStochastic, Fresnel,
                   Default) under a spherical light, and under spotlights (disc emitter with shadows;
                   sphere emitter without shadows beside a soft directional light).
  scene_file/      a scene file (scene.dumb including materials.dumb, meshes in props.obj) that uses
                   presets, groups with fallback / override materials, rotated and scaled items and a
                   rotated spherical-segment camera; render_scene_file.npz holds the reference's renders
                   of it, loaded by the reference's own DumbRenderContext::fromFile (four runs of 512
                   iterations, 32x24).

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


def _obj_text(objects):
    """OBJ text with one `g` group per (name, triangles); x is written negated because the reader
    mirrors it back."""
    lines, base = [], 1
    for name, tris in objects:
        lines.append(f"g {name}")
        for t in tris:
            for v in t:
                lines.append(f"v {-float(v[0]):.9g} {float(v[1]):.9g} {float(v[2]):.9g}")
        for i in range(len(tris)):
            lines.append(f"f {base + 3 * i} {base + 3 * i + 1} {base + 3 * i + 2}")
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


if __name__ == "__main__":
    if not O.reference_available():
        raise SystemExit("build the reference first: bash oracle/build_ref.sh")
    only = sys.argv[1:]
    if not only or "cast" in only:
        cast_fixtures()
    if not only or "render" in only:
        render_fixtures()
    for k in only:
        if k.startswith("render_"):
            render_fixtures(kinds=(k[len("render_"):],))
    if not only or "scene_file" in only:
        scene_file_fixtures()
    print("golden fixtures written to", OUT)
