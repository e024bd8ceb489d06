"""Batched rendering (dr_batch): many scenes of different sizes, resolutions and sample counts in
shared waves, optionally replayed as one CUDA graph.  Every path follows exactly the computation it
has when its scene is rendered alone (same random numbers, same exact cast), so frame buffers agree
with individual dr_render_blocks renders up to the order of float accumulation."""
import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes

pytestmark = pytest.mark.gpu


def _close(a, b, tol=2e-5):
    a = a.cpu().numpy()[:, :3].astype(np.float64)
    b = b.cpu().numpy()[:, :3].astype(np.float64)
    assert np.all(np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-2)), float(np.max(np.abs(a - b)))


def _phys_jobs(cuda):
    rng = np.random.default_rng(3)
    jobs = []
    specs = [(1, 24, 16, (1, 1)), (2, 40, 33, (2, 2)), (3, 64, 48, (3, 3)), (4, 17, 70, (2, 1)), (0, 8, 8, (1, 4))]
    for i, (lvl, W, H, spp) in enumerate(specs):
        room = scenes.box((2, 2, 2), inward=True)
        obj = scenes.displaced_icosphere(lvl, 0.1, i, radius=0.5)
        light = scenes.quad((0.0, 0.999, 0.0), (0.5, 0.5), (0.0, -1.0, 0.0))
        tris = np.concatenate([room, obj, light])
        n = len(tris)
        h = scenes.tri_hash_u32(np.arange(n), i) % 100
        mat = np.where(h < 60, 0, np.where(h < 85, 1, 2)).astype(np.int32)
        sc = dr.Scene(tris, mat_id=mat, materials=[dr.lambert(), dr.mirror(), dr.glossy()])
        emission = np.zeros((n, 3), np.float32)
        emission[-2:] = 10.0
        sc.set_triangle_params(rng.uniform(0.2, 0.8, (n, 3)).astype(np.float32), emission,
                               rng.uniform(0.05, 0.4, n).astype(np.float32))
        cam = dr.camera(dr.LENS_PINHOLE if i % 2 == 0 else dr.LENS_FISHEYE, position=(0.0, 0.0, -0.99),
                        angle=(60.0 if i % 2 == 0 else 170.0, 60.0))
        p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=spp, max_bounces=3 + (i % 3), seed=11 + i)
        nb = dr.block_count(W, H)
        s0, s1 = (0, nb) if i != 3 else (1, nb - 1)
        jobs.append([sc, cam, p, dr.new_frame_buffer(W, H, cuda), s0, s1])
    return jobs


def _render_alone(job, cuda, iteration=1, fb=None):
    sc, cam, p, _, s0, s1 = job
    q = dr.render_params(p.width, p.height, p.mode, (p.samples_x, p.samples_y), p.max_bounces, bool(p.cull_backfaces),
                         p.boxing, iteration, p.seed)
    fb = dr.new_frame_buffer(p.width, p.height, cuda) if fb is None else fb
    r = dr.Renderer(1 << 14)
    r.render_blocks(sc, cam, fb, s0, s1, q)
    torch.cuda.synchronize()
    return fb


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_equals_individual_renders(cuda, use_graph):
    jobs = _phys_jobs(cuda)
    batch = dr.Batch([tuple(j) for j in jobs])
    assert batch.paths() == sum((j[5] - j[4]) * 128 * j[2].samples_x * j[2].samples_y for j in jobs)
    r = dr.Renderer(1 << 13)   # small waves: paths of several jobs share each wave
    batch.render(r, use_graph=use_graph)
    torch.cuda.synchronize()
    for j in jobs:
        _close(j[3], _render_alone(j, cuda))


def test_batch_graph_replay_and_iteration(cuda):
    """A captured graph is replayed; set_iteration moves every job to new samples and blends."""
    jobs = _phys_jobs(cuda)
    batch = dr.Batch([tuple(j) for j in jobs])
    r = dr.Renderer(1 << 15)
    batch.render(r, use_graph=True)
    batch.set_iteration(2)
    batch.render(r, use_graph=True)
    torch.cuda.synchronize()
    for j in jobs:
        fb = _render_alone(j, cuda, iteration=1)
        _render_alone(j, cuda, iteration=2, fb=fb)
        _close(j[3], fb)


def test_reference_mode_batch_with_different_light_counts(cuda):
    room = scenes.box((2, 2, 2), inward=True)
    jobs = []
    for i, nl in enumerate((1, 3)):
        tris = np.concatenate([room, scenes.icosphere(2 + i, 0.5)])
        mat = np.zeros(len(tris), np.int32)
        mat[len(room):] = 1
        mats = [dr.dumb_based(diffuse=(0.7, 0.7, 0.7), metal=0.0), dr.simple_stochastic((0.9, 0.8, 0.7), 0.3, 0.7, 8.0)]
        lights = [dr.spherical_light((1.5, 1.5, 1.5), (0.0, 0.8, 0.0), 0.1),
                  dr.soft_directional_light((0.4, 0.4, 0.6), (0.2, -1.0, 0.1), 3.0, 0.05),
                  dr.directional_light((0.2, 0.3, 0.2), (-0.3, -1.0, 0.2), 3.0)][:nl]
        sc = dr.Scene(tris, mat_id=mat, materials=mats, lights=lights)
        cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.95), angle=60.0)
        W, H = 24 + 8 * i, 20
        p = dr.render_params(W, H, dr.MODE_REFERENCE, samples=(2, 2), max_bounces=2, seed=5 + i)
        jobs.append([sc, cam, p, dr.new_frame_buffer(W, H, cuda), 0, dr.block_count(W, H)])
    batch = dr.Batch([tuple(j) for j in jobs])
    batch.render(dr.Renderer(1 << 12), use_graph=True)
    torch.cuda.synchronize()
    for j in jobs:
        _close(j[3], _render_alone(j, cuda))


def test_batch_rejects_mixed_modes(cuda):
    jobs = _phys_jobs(cuda)[:1]
    room = scenes.box((2, 2, 2), inward=True)
    sc = dr.Scene(room, materials=[dr.dumb_based()], lights=[dr.spherical_light((1, 1, 1), (0, 0.5, 0), 0.1)])
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.9))
    p = dr.render_params(16, 16, dr.MODE_REFERENCE)
    with pytest.raises(dr.DumbRayError):
        dr.Batch([tuple(jobs[0]), (sc, cam, p, dr.new_frame_buffer(16, 16, cuda), 0, 2)])


def test_batch_arena_root_leaf_and_shared_scene(cuda):
    """A scene whose octree is a single root leaf (no nodes) and one scene used by two jobs (stored
    once in the batch's octree arena) render as they do alone."""
    jobs = _phys_jobs(cuda)[:2]
    small = np.concatenate([scenes.quad((0.0, 0.0, 0.5), (1.5, 1.5), (0.0, 0.0, -1.0)),
                            scenes.quad((0.0, 0.9, 0.0), (0.4, 0.4), (0.0, -1.0, 0.0))])
    sc = dr.Scene(small, materials=[dr.lambert()])
    em = np.zeros((4, 3), np.float32)
    em[2:] = 5.0
    sc.set_triangle_params(np.full((4, 3), 0.6, np.float32), em, np.full(4, 0.2, np.float32))
    assert sc.stats()["nodes"] <= 1
    cam = dr.camera(dr.LENS_PINHOLE, position=(0.0, 0.0, -1.0), angle=60.0)
    p = dr.render_params(16, 16, dr.MODE_PHYSICAL, samples=(2, 2), max_bounces=3, seed=4)
    jobs.append([sc, cam, p, dr.new_frame_buffer(16, 16, cuda), 0, dr.block_count(16, 16)])
    shared = jobs[1]
    p2 = dr.render_params(shared[2].width, shared[2].height, dr.MODE_PHYSICAL, samples=(1, 2), max_bounces=2, seed=9)
    jobs.append([shared[0], shared[1], p2, dr.new_frame_buffer(p2.width, p2.height, cuda), 0,
                 dr.block_count(p2.width, p2.height)])
    batch = dr.Batch([tuple(j) for j in jobs])
    batch.render(dr.Renderer(1 << 12), use_graph=True)
    torch.cuda.synchronize()
    for j in jobs:
        _close(j[3], _render_alone(j, cuda))


def test_reference_batch_rejects_mixed_culling(cuda):
    room = scenes.box((2, 2, 2), inward=True)
    sc = dr.Scene(room, materials=[dr.dumb_based()], lights=[dr.spherical_light((1, 1, 1), (0, 0.5, 0), 0.1)])
    cam = dr.camera(dr.LENS_SIMPLE_STOCHASTIC, position=(0.0, 0.0, -0.9))
    a = dr.render_params(16, 16, dr.MODE_REFERENCE, cull_backfaces=True)
    b = dr.render_params(16, 16, dr.MODE_REFERENCE, cull_backfaces=False)
    with pytest.raises(dr.DumbRayError):
        dr.Batch([(sc, cam, a, dr.new_frame_buffer(16, 16, cuda), 0, 2), (sc, cam, b, dr.new_frame_buffer(16, 16, cuda), 0, 2)])
