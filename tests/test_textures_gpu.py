"""Textured reference-mode shading on the GPU (dr_scene_set_textures, ColoredTexture channels).

The kernels follow the CPU oracle's paths with the same random numbers (per-pixel agreement up to
float rounding of transcendentals) and agree statistically with the reference DumbRenderer's renders
of the same textured scenes (golden fixtures render_tex_*.npz)."""
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
import _oracle as O
from _stats import compare_runs

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
from make_golden import texture_scene, TEXTURE_KINDS  # noqa: E402

pytestmark = pytest.mark.gpu


def _scene(kind):
    tris, mat, mats, lights, cam, uv, textures = texture_scene(kind)
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    sc.set_textures(textures, uv)
    return sc, cam, (tris, mat, mats, lights, uv, textures)


def _render(sc, cam, p, cuda):
    fb = dr.new_frame_buffer(p.width, p.height, cuda)
    r = dr.Renderer(1 << 16)
    r.render_blocks(sc, cam, fb, 0, dr.block_count(p.width, p.height), p)
    torch.cuda.synchronize()
    return dr.blockmajor_to_image(fb, p.width, p.height)


@pytest.mark.parametrize("kind", TEXTURE_KINDS)
def test_textured_matches_oracle(cuda, kind):
    sc, cam, (tris, mat, mats, lights, uv, textures) = _scene(kind)
    osc = O.OracleScene(tris, mat_id=mat, materials=mats, lights=lights)
    osc.set_textures(textures, uv)
    p = dr.render_params(40, 30, dr.MODE_REFERENCE, samples=(2, 2), max_bounces=3, seed=6)
    g = _render(sc, cam, p, cuda)[..., :3].astype(np.float64)
    o = dr.blockmajor_to_image(osc.render_blocks(cam, p), 40, 30)[..., :3].astype(np.float64)
    assert np.isfinite(g).all()
    bad = np.abs(g - o) > 2e-3 * np.maximum(np.abs(o), 0.01)
    assert bad.mean() <= 0.02, f"{bad.mean():.4f} of channels differ"
    assert abs(g.mean() - o.mean()) <= 5e-3 * max(abs(o.mean()), 1e-6)


@pytest.mark.parametrize("kind", TEXTURE_KINDS)
def test_textured_matches_reference_statistically(cuda, kind):
    g = np.load(GOLD / f"render_{kind}.npz")
    size, bounces = int(g["size"]), int(g["bounces"])
    sc, cam, _ = _scene(kind)
    runs = []
    for seed in range(300, 308):
        p = dr.render_params(size, size, dr.MODE_REFERENCE, samples=(32, 32), max_bounces=bounces, seed=seed)
        runs.append(_render(sc, cam, p, cuda))
    compare_runs(runs, g["runs"])


def test_texture_errors(cuda):
    tris, mat, mats, lights, cam, uv, textures = texture_scene("tex_diffuse")
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    p = dr.render_params(16, 16, dr.MODE_REFERENCE, samples=(1, 1), max_bounces=1)
    fb = dr.new_frame_buffer(16, 16, cuda)
    r = dr.Renderer(1 << 12)
    with pytest.raises(dr.DumbRayError):       # materials use textures that were not set
        r.render_blocks(sc, cam, fb, 0, dr.block_count(16, 16), p)
    with pytest.raises(dr.DumbRayError):       # texture index beyond the textures given
        sc.set_textures(textures[:1], uv)
    sc.set_textures(textures, uv)
    r.render_blocks(sc, cam, fb, 0, dr.block_count(16, 16), p)
    torch.cuda.synchronize()
    assert torch.isfinite(fb).all()
