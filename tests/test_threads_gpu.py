"""Concurrent callers, the way the reference's BlockRenderer makes them (BlockRenderer.cu:74-97): one
host thread per (GPU, thread slot), each with its own renderer and stream, rendering disjoint block
ranges of one frame buffer over one shared, read-only scene.  ctypes releases the GIL around every
library call, so the threads' calls overlap inside the library.  Each thread's blocks must equal a
single-threaded render of the same blocks (up to float accumulation order: the accumulators take
atomic adds), and casts from several threads must equal a single-threaded cast exactly."""
import sys
import threading
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

THREADS = 4


def _run_threads(fns):
    errors = []
    start = threading.Barrier(len(fns))

    def wrap(f):
        try:
            start.wait(timeout=60)
            f()
        except BaseException as e:  # reported in the main thread
            errors.append(e)

    ts = [threading.Thread(target=wrap, args=(f,)) for f in fns]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in ts), "a rendering thread did not finish"
    if errors:
        raise errors[0]


def _iterations(rend, sc, cam, fb, start, end, p, n_iter, stream=None):
    for it in range(1, n_iter + 1):
        p.iteration = it
        rend.render_blocks(sc, cam, fb, start, end, p, stream)


def _threaded_vs_single(sc, cam, p, cuda, n_iter=3, wave=2048, lanes=2):
    nb = dr.block_count(p.width, p.height)
    one = dr.new_frame_buffer(p.width, p.height, cuda)
    _iterations(dr.Renderer(wave, 1), sc, cam, one, 0, nb, p, n_iter)
    torch.cuda.synchronize()
    fb = dr.new_frame_buffer(p.width, p.height, cuda)
    cuts = [nb * k // THREADS for k in range(THREADS + 1)]
    renderers = [dr.Renderer(wave, lanes) for _ in range(THREADS)]
    streams = [torch.cuda.Stream() for _ in range(THREADS)]
    torch.cuda.synchronize()   # the frame buffer's zero fill ran on this thread's stream

    def job(k):
        def run():
            q = dr.DrRenderParams.from_buffer_copy(p)
            _iterations(renderers[k], sc, cam, fb, cuts[k], cuts[k + 1], q, n_iter, streams[k])
            streams[k].synchronize()
        return run

    _run_threads([job(k) for k in range(THREADS)])
    torch.cuda.synchronize()
    got, want = fb.cpu().numpy(), one.cpu().numpy()
    assert np.isfinite(got).all() and got[..., :3].any()
    assert np.allclose(got, want, rtol=1e-4, atol=1e-6)


def test_threads_render_disjoint_blocks_physical(cuda):
    S = scenes.box_and_icosphere(3)
    mats = [dr.lambert((0.7, 0.7, 0.7)), dr.lambert((0.7, 0.1, 0.1)), dr.lambert((0.0, 0.0, 0.0), emission=(10.0, 10.0, 10.0))]
    sc = dr.Scene(S["tris"], mat_id=S["mat_id"], materials=mats)
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -0.9), target=(0.0, 0.0, 0.0), angle=(60.0, 60.0))
    p = dr.render_params(128, 96, dr.MODE_PHYSICAL, samples=(2, 2), max_bounces=4, seed=5)
    _threaded_vs_single(sc, cam, p, cuda)


def test_threads_render_disjoint_blocks_reference_mode(cuda):
    tris, mat, mats, lights, cam = render_scene("spot")
    lights = lights + render_scene("diffuse")[3]
    sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
    p = dr.render_params(96, 64, dr.MODE_REFERENCE, samples=(2, 2), max_bounces=3, seed=6)
    _threaded_vs_single(sc, cam, p, cuda)


def test_threads_cast_concurrently(cuda):
    sc = dr.Scene(scenes.displaced_icosphere(5, seed=3))
    lo, hi = (-1.2, -1.2, -1.2), (1.2, 1.2, 1.2)
    rays = [scenes.incoherent_rays(60_000, lo, hi, seed=10 + k) for k in range(THREADS)]
    rays = [(torch.from_numpy(np.ascontiguousarray(o, np.float32)).to(cuda),
             torch.from_numpy(np.ascontiguousarray(d, np.float32)).to(cuda)) for (o, d) in rays]
    want = [dr.cast(sc, o, d) for (o, d) in rays]
    torch.cuda.synchronize()
    want = [(t.cpu().numpy(), h.cpu().numpy()) for (t, h) in want]
    got = [None] * THREADS
    streams = [torch.cuda.Stream() for _ in range(THREADS)]

    def job(k):
        def run():
            res = [dr.cast(sc, *rays[k], stream=streams[k]) for _ in range(3)]
            streams[k].synchronize()
            got[k] = [(t.cpu().numpy(), h.cpu().numpy()) for (t, h) in res]
        return run

    _run_threads([job(k) for k in range(THREADS)])
    for k in range(THREADS):
        for (t, h) in got[k]:
            assert np.array_equal(t, want[k][0])
            assert np.array_equal(h, want[k][1])
