"""Scene files rendered on the GPU.

The committed fixture (tests/golden/scene_file: includes, presets, groups with fallback / override
materials, rotated and scaled items, a rotated spherical-segment camera whose lens origins take the
reference's point-transform rows) is loaded by dr_scene_file_load and rendered by dr_render_blocks:
  * against the CPU oracle with the same counter-based random numbers (per-pixel agreement up to
    float rounding of transcendentals, as in the other reference-mode tests);
  * against the reference DumbRenderer's renders of the same file loaded by the reference's own
    DumbRenderContext::fromFile (golden fixture), statistically."""
from pathlib import Path

import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
import _oracle as O
from _stats import compare_runs

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
SCENE = GOLD / "scene_file" / "scene.dumb"


def _render(scene, cam, p, cuda):
    fb = dr.new_frame_buffer(p.width, p.height, cuda)
    r = dr.Renderer(1 << 16)
    r.render_blocks(scene, cam, fb, 0, dr.block_count(p.width, p.height), p)
    torch.cuda.synchronize()
    return dr.blockmajor_to_image(fb, p.width, p.height)


def test_scene_file_matches_oracle(cuda):
    f = dr.load_scene_file(SCENE)
    assert f.camera.origin_rows == 1 and f.camera.lens == dr.LENS_SPHERICAL_SEGMENT
    sc = f.scene()
    osc = O.OracleScene(f.tris, normals=f.normals, mat_id=f.mat_id, materials=f.materials, lights=f.lights)
    p = f.render_params(40, 30, seed=11)
    p.samples_x, p.samples_y = 2, 2
    gpu = _render(sc, f.camera, p, cuda)
    ora = dr.blockmajor_to_image(osc.render_blocks(f.camera, p), 40, 30)
    g, o = gpu[..., :3].astype(np.float64), ora[..., :3].astype(np.float64)
    assert np.isfinite(g).all()
    bad = np.abs(g - o) > 2e-3 * np.maximum(np.abs(o), 0.01)
    assert bad.mean() <= 0.02, f"{bad.mean():.4f} of channels differ"
    assert abs(g.mean() - o.mean()) <= 5e-3 * max(abs(o.mean()), 1e-6)


def test_origin_rows_change_the_spherical_segment_rays(cuda):
    """The same camera with origin_rows = 0 (origins through the direction basis) renders a
    different image: the rows are what the reference's Camera applies to lens origins."""
    f = dr.load_scene_file(SCENE)
    sc = f.scene()
    p = f.render_params(24, 18, seed=2)
    a = _render(sc, f.camera, p, cuda)
    cam = dr.DrCamera.from_buffer_copy(f.camera)
    cam.origin_rows = 0
    b = _render(sc, cam, p, cuda)
    assert not np.array_equal(a, b)


def test_scene_file_matches_reference_renderer_statistically(cuda):
    """8 GPU runs (1024 samples per pixel each) vs the reference's 4 runs of 512 iterations of the
    file as the reference loads it."""
    g = np.load(GOLD / "render_scene_file.npz")
    W, H = int(g["width"]), int(g["height"])
    f = dr.load_scene_file(SCENE)
    sc = f.scene()
    runs = []
    for seed in range(200, 208):
        p = f.render_params(W, H, seed=seed)
        p.samples_x, p.samples_y = 32, 32
        runs.append(_render(sc, f.camera, p, cuda))
    compare_runs(runs, g["runs"])


def test_create_scene_through_the_c_abi(cuda):
    """dr_scene_file_create_scene builds the same octree as a Scene over the exported arrays."""
    import ctypes
    L = dr.lib()
    f = dr.load_scene_file(SCENE)
    h = ctypes.c_void_p()
    dr.check(L.dr_scene_file_load(str(SCENE).encode(), ctypes.byref(h)))
    try:
        s = ctypes.c_void_p()
        bp = dr.DrBuildParams(0, 0, 0, 0.0, 0)
        dr.check(L.dr_scene_file_create_scene(h, ctypes.byref(bp), ctypes.byref(s)))
        try:
            import ctypes as C
            n, lv, rf, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
            dr.check(L.dr_scene_stats(s, C.byref(n), C.byref(lv), C.byref(rf), C.byref(d)))
            assert dict(nodes=n.value, leaves=lv.value, refs=rf.value, depth=d.value) == f.scene().stats()
        finally:
            L.dr_scene_destroy(s)
    finally:
        L.dr_scene_file_destroy(h)


TEX_SCENE = GOLD / "scene_file_tex" / "scene.dumb"


def test_textured_scene_file_matches_oracle(cuda):
    f = dr.load_scene_file(TEX_SCENE)
    assert len(f.textures) == 4
    sc = f.scene()
    osc = O.OracleScene(f.tris, normals=f.normals, mat_id=f.mat_id, materials=f.materials, lights=f.lights)
    osc.set_textures(f.textures, f.uv)
    p = f.render_params(40, 40, seed=4)
    p.samples_x, p.samples_y = 2, 2
    g = _render(sc, f.camera, p, cuda)[..., :3].astype(np.float64)
    o = dr.blockmajor_to_image(osc.render_blocks(f.camera, p), 40, 40)[..., :3].astype(np.float64)
    bad = np.abs(g - o) > 2e-3 * np.maximum(np.abs(o), 0.01)
    assert bad.mean() <= 0.02, f"{bad.mean():.4f} of channels differ"
    assert abs(g.mean() - o.mean()) <= 5e-3 * max(abs(o.mean()), 1e-6)


def test_textured_scene_file_matches_reference_renderer_statistically(cuda):
    g = np.load(GOLD / "render_scene_file_tex.npz")
    W, H = int(g["width"]), int(g["height"])
    f = dr.load_scene_file(TEX_SCENE)
    sc = f.scene()
    runs = []
    for seed in range(400, 408):
        p = f.render_params(W, H, seed=seed)
        p.samples_x, p.samples_y = 32, 32
        runs.append(_render(sc, f.camera, p, cuda))
    compare_runs(runs, g["runs"])
