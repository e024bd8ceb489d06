"""Generates the golden fixtures in tests/golden/ by running the REFERENCE DumbRay host path
(oracle/_ref/libdumbref.so, compiled from the reference sources by oracle/build_ref.sh).

  cast_small.npz   displaced icosphere level 4 + inward 3x3x3 box (5,132 tris); 8,192 incoherent rays
                   and 64x48 pinhole primaries; reference Octree::cast hit index and t, culling on and
                   off; reference node count.
  cast_c1.npz      the 20,492-triangle box + icosphere level 5 geometry; 16,384 incoherent rays,
                   culling on.
  render_*.npz     reference DumbRenderer CPU renders (four independent runs of 512 progressive
                   iterations each) of small reference-expressible scenes, 32x32.

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
    if kind == "diffuse":
        obj = dr.dumb_based(diffuse=(0.5, 0.6, 0.7), metal=0.0)
    elif kind == "metal":
        obj = dr.dumb_based(fresnel=(1.022, 0.782, 0.344), specular=16.0, diffuse=(1.0, 1.0, 1.0), metal=0.5)
    else:
        obj = dr.simple_stochastic((0.9, 0.9, 0.9), 0.3, 0.7, 8.0)
    mats = [white, red, obj]
    lights = [dr.spherical_light((1.5, 1.5, 1.5), (0.0, 0.8, 0.0), 0.1)]
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.95), angle=60.0)
    return tris, mat, mats, lights, cam


def render_fixtures(iterations=512, runs=4, size=32, bounces=2):
    for kind in ("diffuse", "metal", "ss"):
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


if __name__ == "__main__":
    if not O.reference_available():
        raise SystemExit("build the reference first: bash oracle/build_ref.sh")
    cast_fixtures()
    render_fixtures()
    print("golden fixtures written to", OUT)
