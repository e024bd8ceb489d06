"""dr_render_blocks_noalloc against dr_render_blocks.

The allocation-free entry point serves callers that cannot allocate device memory while they
render (under another owner's memory pool or fixed budget, or on a thread where cudaMalloc's
implicit device synchronisation is not acceptable).  It must produce the same frame
buffer as the regular entry point - same paths, same blending - on consecutive calls, which share
(and must correctly re-clear) its fixed scratch array.  Tolerance: the same per-pixel comparison
as the other render tests (accumulation order of float atomics may differ).

Collected last on purpose, so a run that stops at the first failure has run every other test."""
import ctypes

import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes

pytestmark = pytest.mark.gpu


def _compare(gpu, ref, tol_rel=2e-3, max_bad_frac=0.02):
    gpu = gpu[..., :3].astype(np.float64)
    ref = ref[..., :3].astype(np.float64)
    assert np.isfinite(gpu).all()
    bad = np.abs(gpu - ref) > tol_rel * np.maximum(np.abs(ref), 0.01)
    assert bad.mean() <= max_bad_frac, f"{bad.mean():.4f} of channels differ"


def _scene(kind):
    """(scene, camera, mode) of each covered case: reference semantics with a sphere light and a soft
    directional light (SimpleStochastic lens), the same room through the spherical-segment lens, a
    spotlight room (16-photon disc emitter with shadows), and the physical mode."""
    room = scenes.box((2, 2, 2), inward=True)
    sph = scenes.icosphere(3, 0.5)
    tris = np.concatenate([room, sph])
    mat = np.zeros(len(tris), np.int32)
    mat[len(room):] = 1
    if kind != "physical":
        mats = [dr.dumb_based(diffuse=(0.7, 0.7, 0.7), metal=0.0), dr.simple_stochastic((0.9, 0.8, 0.7), 0.3, 0.7, 8.0)]
        lights = [dr.spherical_light((1.5, 1.5, 1.5), (0.0, 0.8, 0.0), 0.1),
                  dr.soft_directional_light((0.4, 0.4, 0.6), (0.2, -1.0, 0.1), 3.0, 0.05)]
        cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.95), angle=60.0)
        if kind == "segment_lens":
            cam = dr.camera(dr.LENS_SPHERICAL_SEGMENT, position=(0.0, 0.0, -0.95), angle=(70.0, 50.0),
                            focal_distance=2.0, softness=0.01, filter=(1.0, 0.9, 0.8))
        elif kind == "spotlight":
            lights = [dr.spotlight((1.0, 0.95, 0.9), 150.0, (0.3, 0.7, -0.4), (-0.2, -1.0, 0.3), 20.0, 50.0, 2.0, 0.15,
                                   emit_from_sphere=False, cast_shadows=True, samples=16)]
        return dr.Scene(tris, mat_id=mat, materials=mats, lights=lights), cam, dr.MODE_REFERENCE
    c = scenes.box_and_icosphere(3)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.glossy((0.8, 0.6, 0.4), 0.2),
            dr.lambert((0.0, 0.0, 0.0), emission=(10.0, 10.0, 10.0))]
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    return dr.Scene(c["tris"], mat_id=c["mat_id"], materials=mats), cam, dr.MODE_PHYSICAL


@pytest.mark.parametrize("kind", ["reference", "segment_lens", "spotlight", "physical"])
def test_noalloc_matches_render_blocks_on_consecutive_calls(kind):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda:0")
    scene, cam, mode = _scene(kind)
    W, H = 72, 40
    nb = dr.block_count(W, H)
    fb_ref = dr.new_frame_buffer(W, H, dev)
    fb_new = dr.new_frame_buffer(W, H, dev)
    r = dr.Renderer(1 << 16)
    # two calls in a row on the same frame buffers: a set (iteration 1) then a blend (iteration 2)
    for it in (1, 2):
        p = dr.render_params(W, H, mode, samples=(2, 2), max_bounces=3, iteration=it, seed=21)
        r.render_blocks(scene, cam, fb_ref, 1, nb, p)
        dr.render_blocks_noalloc(scene, cam, fb_new, 1, nb, p)
        torch.cuda.synchronize()
        a = dr.blockmajor_to_image(fb_ref, W, H)
        b = dr.blockmajor_to_image(fb_new, W, H)
        _compare(b, a)
        assert np.array_equal(fb_new[:128].cpu().numpy(), np.zeros((128, 4), np.float32))  # block 0 untouched


def test_noalloc_rejects_ranges_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda:0")
    scene, cam, _ = _scene("reference")
    W, H = 1024, 512   # 4096 blocks > DR_NOALLOC_MAX_BLOCKS
    fb = dr.new_frame_buffer(W, H, dev)
    p = dr.render_params(W, H, dr.MODE_REFERENCE)
    with pytest.raises(dr.DumbRayError) as ei:
        dr.render_blocks_noalloc(scene, cam, fb, 0, dr.block_count(W, H), p)
    assert ei.value.status == dr.DR_E_CAPACITY
    assert "at most 2048" in str(ei.value)
