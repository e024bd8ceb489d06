"""Concurrent wave pipelines ("lanes") of one render (dr_renderer_set_lanes).

A render's waves alternate over the lanes, each with its own queues and stream, adding into one
accumulator; the image must not depend on the lane count beyond float accumulation order (the
accumulator takes atomic adds from every lane).  Small waves force many waves per render so that
every lane gets work."""
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
from make_golden import render_scene  # noqa: E402

pytestmark = pytest.mark.gpu


def _physical():
    S = scenes.box_and_icosphere(3)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.lambert((0.7, 0.1, 0.1)), dr.lambert((0.0, 0.0, 0.0), emission=(10.0, 10.0, 10.0))]
    sc = dr.Scene(S["tris"], mat_id=S["mat_id"], materials=mats)
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.9), target=(0.0, 0.0, 0.0), angle=(60.0, 60.0))
    return sc, cam


def _render(rend, sc, cam, p, cuda, start=0, end=None):
    nb = dr.block_count(p.width, p.height)
    fb = dr.new_frame_buffer(p.width, p.height, cuda)
    rend.render_blocks(sc, cam, fb, start, nb if end is None else end, p)
    torch.cuda.synchronize()
    return fb.cpu().numpy()


@pytest.mark.parametrize("lanes", [2, 3, 8])
def test_lanes_match_one_lane_physical(cuda, lanes):
    sc, cam = _physical()
    p = dr.render_params(96, 64, dr.MODE_PHYSICAL, samples=(2, 4), max_bounces=4, seed=3)
    one = _render(dr.Renderer(4096, 1), sc, cam, p, cuda)
    r = dr.Renderer(4096, lanes)
    assert r.lanes == lanes
    many = _render(r, sc, cam, p, cuda)
    assert np.allclose(many, one, rtol=1e-4, atol=1e-6)
    # a block range that is not the whole frame
    nb = dr.block_count(96, 64)
    part = _render(r, sc, cam, p, cuda, 5, nb - 7)
    assert np.allclose(part[5 * 128:(nb - 7) * 128], one[5 * 128:(nb - 7) * 128], rtol=1e-4, atol=1e-6)
    assert not part[:5 * 128].any() and not part[(nb - 7) * 128:].any()


def test_lanes_match_one_lane_reference_mode(cuda):
    """Reference mode: photon casts (continuing through blockers in place), per lane."""
    tris, mat, mats, lights, cam = render_scene("spot")
    lights = lights + render_scene("diffuse")[3]
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    p = dr.render_params(64, 48, dr.MODE_REFERENCE, samples=(2, 2), max_bounces=3, seed=8)
    one = _render(dr.Renderer(2048, 1), sc, cam, p, cuda)
    many = _render(dr.Renderer(2048, 4), sc, cam, p, cuda)
    assert np.allclose(many, one, rtol=1e-4, atol=1e-6)


def test_lanes_in_a_captured_batch(cuda):
    """A batch graph captured with several lanes (their streams join the capture through events)
    renders what a one-lane graph renders, and replays."""
    sc, cam = _physical()
    fbs = {}
    for lanes in (1, 3):
        fbs[lanes] = [dr.new_frame_buffer(w, h, cuda) for (w, h) in ((64, 64), (48, 80), (32, 32))]
    out = {}
    for lanes in (1, 3):
        items = []
        for k, (w, h) in enumerate(((64, 64), (48, 80), (32, 32))):
            p = dr.render_params(w, h, dr.MODE_PHYSICAL, samples=(2, 2), max_bounces=3, seed=20 + k)
            items.append((sc, cam, p, fbs[lanes][k], 0, dr.block_count(w, h)))
        b = dr.Batch(items)
        r = dr.Renderer(2048, lanes)
        b.render(r, use_graph=True)
        b.set_iteration(2)
        b.render(r, use_graph=True)
        torch.cuda.synchronize()
        out[lanes] = [fb.cpu().numpy() for fb in fbs[lanes]]
        b.close()
        r.close()
    for a, c in zip(out[1], out[3]):
        assert np.allclose(a, c, rtol=1e-4, atol=1e-6)


def test_busy_time_and_arguments(cuda):
    sc, cam = _physical()
    p = dr.render_params(128, 96, dr.MODE_PHYSICAL, samples=(2, 2), max_bounces=3, seed=1)
    for lanes in (1, 4):
        r = dr.Renderer(4096, lanes)
        r.set_profiling(True)
        _render(r, sc, cam, p, cuda)
        t = r.kernel_times()
        busy = r.kernel_busy()
        r.set_profiling(False)
        for k, (ms, n) in t.items():
            assert n > 0 and busy[k] > 0.0
            assert busy[k] <= ms * (1 + 1e-6) + 1e-3
            if lanes == 1:
                assert busy[k] == pytest.approx(ms, rel=1e-4, abs=1e-3)
    r = dr.Renderer(4096)
    assert r.lanes == 4
    for bad in (0, 9, -1):
        with pytest.raises(dr.DumbRayError):
            r.set_lanes(bad)


@pytest.mark.parametrize("mode", [dr.MODE_PHYSICAL, dr.MODE_REFERENCE])
def test_block_shapes_render_the_same_image(cuda, mode):
    """dr_renderer_set_block_shape changes how the traversal kernels are launched, not what they
    compute: both shapes give the same image (up to float accumulation order), also through a
    captured batch graph, which is re-captured when the shape changes."""
    if mode == dr.MODE_PHYSICAL:
        sc, cam = _physical()
    else:
        tris, mat, mats, lights, cam = render_scene("metal")
        sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    p = dr.render_params(96, 64, mode, samples=(2, 2), max_bounces=4, seed=12)
    r = dr.Renderer(4096, 2)
    assert r.block_shape == 0
    a = _render(r, sc, cam, p, cuda)
    r.set_block_shape(1)
    assert r.block_shape == 1
    b = _render(r, sc, cam, p, cuda)
    assert np.allclose(a, b, rtol=1e-4, atol=1e-6)
    fb = dr.new_frame_buffer(96, 64, cuda)
    batch = dr.Batch([(sc, cam, p, fb, 0, dr.block_count(96, 64))])
    for shape in (0, 1, 0):
        r.set_block_shape(shape)
        fb.zero_()
        batch.render(r, use_graph=True)
        torch.cuda.synchronize()
        assert np.allclose(fb.cpu().numpy(), a, rtol=1e-4, atol=1e-6)
    with pytest.raises(dr.DumbRayError):
        r.set_block_shape(2)
    batch.close()


def test_wave_counts_sum_to_the_counted_rays(cuda):
    """dr_renderer_wave_counts: with one lane and a wave that holds the whole render, the per-bounce
    queue sizes of the last wave are the render's own, so the extension rays add up to what the
    counting pass counts and bounce 0 holds one camera ray per path."""
    sc, cam = _physical()
    p = dr.render_params(96, 64, dr.MODE_PHYSICAL, samples=(2, 2), max_bounces=4, seed=3)
    r = dr.Renderer(1 << 16, 1)
    r.set_counting(True)
    _render(r, sc, cam, p, cuda)
    cnt = r.counters()
    rays, shadows = r.wave_counts(6)
    assert rays[0] == 96 * 64 * 4
    assert sum(rays) == cnt["trace_rays"]
    assert sum(shadows) == cnt["shadow_casts"]
    assert rays[5] == 0 and all(a >= b for a, b in zip(rays, rays[1:]))
    with pytest.raises(dr.DumbRayError):
        r.wave_counts(69)
