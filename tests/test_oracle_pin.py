"""The oracle is pinned to the reference: bit-exact casts against golden vectors produced by the
reference's own Octree::cast, and renders statistically equal to the reference DumbRenderer."""
from pathlib import Path

import numpy as np
import pytest

import dumbray_gb300 as dr
import _oracle as O

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("fixture,culls", [("cast_small.npz", (1, 0)), ("cast_c1.npz", (1,))])
def test_oracle_cast_matches_reference_golden(fixture, culls):
    g = np.load(GOLD / fixture)
    osc = O.OracleScene(g["tris"])
    assert osc.node_count() == int(g["nodes"])
    for cull in culls:
        idx, t, _, _ = osc.cast(g["o"], g["d"], cull=bool(cull))
        ref_idx, ref_t = g[f"idx_cull{cull}"], g[f"t_cull{cull}"]
        assert np.array_equal(idx, ref_idx)
        hit = ref_idx >= 0
        assert np.array_equal(t[hit].view(np.int32), ref_t[hit].view(np.int32))  # bit-exact t


def test_oracle_cast_matches_reference_golden_level8():
    """The ray-cast microbenchmark mesh itself (level-8 displaced icosphere, 1,310,720 triangles) on the
    reference's octree: node count and the reference's hits (index and t bit-exact) on the golden
    subset of the benchmark's rays, culling on and off."""
    sys_path_golden()
    from make_golden import c2_rays, mesh_sha256
    from dumbray_gb300 import scenes
    g = np.load(GOLD / "cast_c2_l8.npz")
    tris = scenes.displaced_icosphere(8, 0.1, 1)
    assert mesh_sha256(tris) == str(g["mesh_sha256"])
    o, d = c2_rays()
    assert np.array_equal(o, g["o"]) and np.array_equal(d, g["d"])
    osc = O.OracleScene(tris)
    assert osc.node_count() == int(g["nodes"])
    for cull in (1, 0):
        idx, t, _, _ = osc.cast(o, d, cull=bool(cull))
        ref_idx, ref_t = g[f"idx_cull{cull}"], g[f"t_cull{cull}"]
        assert np.array_equal(idx, ref_idx)
        hit = ref_idx >= 0
        assert np.array_equal(t[hit].view(np.int32), ref_t[hit].view(np.int32))


@pytest.mark.skipif(not O.reference_available(), reason="reference library not built here")
def test_oracle_cast_matches_live_reference():
    from dumbray_gb300 import scenes
    tris = np.concatenate([scenes.displaced_icosphere(3, 0.15, 4), scenes.box((2.5, 2.5, 2.5), inward=True)])
    o, d = scenes.incoherent_rays(20000, -1.1, 1.1, seed=2)
    d[::7, 0] = 0.0  # axis-parallel components exercise the infinite inverse direction
    d[::11, 1] = -0.0
    for cull in (True, False):
        ri, rt, nodes = O.ref_cast(tris, o, d, cull=cull)
        osc = O.OracleScene(tris)
        oi, ot, _, _ = osc.cast(o, d, cull=cull)
        assert osc.node_count() == nodes
        assert np.array_equal(oi, ri)
        assert np.array_equal(ot[ri >= 0].view(np.int32), rt[ri >= 0].view(np.int32))



@pytest.mark.parametrize("kind", ["diffuse", "metal", "ss", "fresnel", "default", "spot", "spot_open"])
def test_oracle_render_matches_reference_statistically(kind):
    """4 oracle runs (256 spp each) vs 4 reference DumbRenderer runs (512 iterations each): MSE of
    the run means within 1.5x of what the runs' own per-pixel variances predict; image means within
    4 standard errors (see _stats.compare_runs)."""
    sys_path_golden()
    from make_golden import render_scene
    from _stats import compare_runs
    g = np.load(GOLD / f"render_{kind}.npz")
    size, bounces = int(g["size"]), int(g["bounces"])
    tris, mat, mats, lights, cam = render_scene(kind)
    osc = O.OracleScene(tris, mat_id=mat, materials=mats, lights=lights)
    runs = []
    for seed in (1, 2, 3, 4):
        p = dr.render_params(size, size, dr.MODE_REFERENCE, samples=(16, 16), max_bounces=bounces, seed=seed)
        runs.append(dr.blockmajor_to_image(osc.render_blocks(cam, p), size, size))
    compare_runs(runs, g["runs"])


def sys_path_golden():
    import sys
    p = str(GOLD)
    if p not in sys.path:
        sys.path.insert(0, p)


@pytest.mark.parametrize("kind", ["tex_diffuse", "tex_normal", "tex_alpha", "tex_fresnel"])
def test_oracle_textured_render_matches_reference_statistically(kind):
    """Textured scenes (ColoredTexture channels with tiling / offset, nearest and bilinear texture
    filtering, a normal map, an alpha cutout, a textured Fresnel shader): 4 oracle runs vs the 4
    reference runs of the golden fixture."""
    sys_path_golden()
    from make_golden import texture_scene
    from _stats import compare_runs
    g = np.load(GOLD / f"render_{kind}.npz")
    size, bounces = int(g["size"]), int(g["bounces"])
    tris, mat, mats, lights, cam, uv, textures = texture_scene(kind)
    osc = O.OracleScene(tris, mat_id=mat, materials=mats, lights=lights)
    osc.set_textures(textures, uv)
    runs = []
    for seed in (1, 2, 3, 4):
        p = dr.render_params(size, size, dr.MODE_REFERENCE, samples=(16, 16), max_bounces=bounces, seed=seed)
        runs.append(dr.blockmajor_to_image(osc.render_blocks(cam, p), size, size))
    compare_runs(runs, g["runs"])
