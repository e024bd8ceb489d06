"""Progressive render process (dr_progressive): a native worker thread rendering iteration after
iteration, checked against the same iterations rendered directly with dr_render_blocks (same random
numbers; images equal up to the order of per-pixel float accumulation, 2e-5 relative)."""
import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes

pytestmark = pytest.mark.gpu

W, H = 40, 36


def _scene():
    c = scenes.box_and_icosphere(3)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.lambert((0.7, 0.1, 0.1)), dr.lambert((0.0, 0.0, 0.0), emission=(10.0, 10.0, 10.0))]
    return dr.Scene(c["tris"], mat_id=c["mat_id"], materials=mats, box_epsilon=dr.PHYSICAL_TREE)


def _direct(sc, cam, p, iterations, cuda, seed=None):
    fb = dr.new_frame_buffer(W, H, cuda)
    r = dr.Renderer(0)
    for it in iterations:
        q = dr.render_params(W, H, dr.MODE_PHYSICAL, (p.samples_x, p.samples_y), p.max_bounces, True, p.boxing, it,
                             p.seed if seed is None else seed)
        r.render_blocks(sc, cam, fb, 0, dr.block_count(W, H), q)
    torch.cuda.synchronize()
    return dr.image_from_blocks(fb, W, H)


def _close(a, b, tol=2e-5):
    assert np.all(np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-2)), float(np.max(np.abs(a - b)))


def test_progressive_accumulates_like_direct_iterations(cuda, tmp_path):
    sc = _scene()
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(2, 2), max_bounces=4, seed=21)
    P = dr.Progressive(sc, cam, p)
    calls = {"it": 0, "done": 0, "err": 0}
    P.set_callbacks(lambda: calls.__setitem__("it", calls["it"] + 1), lambda: calls.__setitem__("done", calls["done"] + 1),
                    lambda: calls.__setitem__("err", calls["err"] + 1))
    P.set_target(4)
    P.start()
    P.wait(4)
    img, it = P.read()
    assert it == 4 and P.completed() == 4
    _close(img, _direct(sc, cam, p, [1, 2, 3, 4], cuda))
    P.save_png(tmp_path / "p.png")
    assert (tmp_path / "p.png").stat().st_size > 4 * W * H
    # a new view restarts the accumulation
    cam2 = dr.camera(dr.LENS_FISHEYE, position=(0.0, 0.0, -0.99), angle=(170.0, 170.0))
    P.set_target(2)
    P.set_view(cam=cam2)
    P.wait(2)
    P.stop()
    img2, it2 = P.read()
    assert it2 == 2
    _close(img2, _direct(sc, cam2, p, [1, 2], cuda))
    assert calls["it"] >= 6 and calls["done"] >= 2 and calls["err"] == 0
    assert P.render_seconds() > 0
    P.close()


def test_double_buffered_frames_are_fresh_single_iterations(cuda):
    sc = _scene()
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.99), angle=60.0)
    p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(1, 2), max_bounces=3, seed=5)
    P = dr.Progressive(sc, cam, p, double_buffered=True)
    P.set_target(3)
    P.start()
    P.wait(3)
    P.stop()
    img, it = P.read()
    assert it == 1
    # frames 0, 1, 2 were rendered with seeds seed + frame * 0x9E3779B9; the last one is published
    _close(img, _direct(sc, cam, p, [1], cuda, seed=(5 + 2 * 0x9E3779B9) & 0xFFFFFFFF))
    P.close()


def test_render_errors_reach_the_error_callback(cuda):
    sc = _scene()
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.99))   # a reference lens in the physical mode
    p = dr.render_params(W, H, dr.MODE_PHYSICAL)
    P = dr.Progressive(sc, cam, p)
    errs = []
    P.set_callbacks(on_error=lambda: errs.append(1))
    P.set_target(1)
    P.start()
    with pytest.raises(dr.DumbRayError):
        P.wait(1, timeout_ms=500)
    P.stop()
    assert errs
    with pytest.raises(dr.DumbRayError):
        P.read()
    P.close()
