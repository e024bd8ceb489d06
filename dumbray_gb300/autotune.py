"""Autotuner for batched rendering.

Picks, by timing short renders on the GPU:
  * the octree leaf split threshold (the maximum triangle count of a leaf before it is split) per
    scene-size class, for physical-mode scenes.  The reference fixes it at 8
    (__source__/DataStructures/Objects/Scene/Raycasters/Octree/Octree.cuh, OCTREE_POLYCOUNT_TO_SPLIT_NODE);
    a reference-mode scene keeps 8 because its casts must match the reference tree bit for bit.
    Larger leaves trade child-box tests for triangle tests, which the cooperative warp-wide leaf
    rounds run well, so the best value depends on the triangle density of the scene.
  * the wave size (paths in flight per wave = queue capacity of the renderer) of a batch;
  * the block shape of the traversal kernels (256 threads x 3 blocks or 128 x 6 per SM).

Each probe is timed with CUDA events after one untimed render; the measured table is returned
with the choice so callers can report it.
"""
from __future__ import annotations

import math
import time

import numpy as np

SIZE_CLASSES = (10_000, 100_000, 1_000_000)   # class k holds scenes with tris < SIZE_CLASSES[k]


def size_class(n_tris: int) -> int:
    for k, lim in enumerate(SIZE_CLASSES):
        if n_tris < lim:
            return k
    return len(SIZE_CLASSES)


def _time_ms(fn, reps: int = 2) -> float:
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_leaf_threshold(make_scene, scenes_by_class, camera_for, probe=(512, 512, 4), depth=6,
                        candidates=(3, 4, 6, 8, 12), device="cuda"):
    """make_scene(job, split_threshold) -> dr.Scene; scenes_by_class: {class: job} representative
    jobs; camera_for(job) -> dr camera.  Renders a probe frame (width, height, spp) of every
    representative with each candidate threshold; returns ({class: best}, {class: {cand: ms}})."""
    import dumbray_gb300 as dr

    W, H, spp = probe
    sx = int(round(math.sqrt(spp)))
    sy = max(1, spp // sx)
    best, table = {}, {}
    rend = dr.Renderer(1 << 22)
    fb = dr.new_frame_buffer(W, H, device)
    nb = dr.block_count(W, H)
    for cls, job in sorted(scenes_by_class.items()):
        table[cls] = {}
        cam = camera_for(job)
        p = dr.render_params(W, H, dr.MODE_PHYSICAL, samples=(sx, sy), max_bounces=depth, seed=99)
        for c in candidates:
            sc = make_scene(job, c)
            table[cls][c] = round(_time_ms(lambda: rend.render_blocks(sc, cam, fb, 0, nb, p)), 3)
            sc.close()
        best[cls] = min(table[cls], key=table[cls].get)
    rend.close()
    return best, table


def tune_wave(batch, candidates=(1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24), use_graph=True, lanes=0):
    """Times one batch render per candidate wave size; returns (best, {wave: ms}, renderer of the best).
    Candidates above the batch's path count are skipped (a wave never exceeds the batch).  ``lanes``:
    concurrent wave pipelines of the renderers (0 = library default)."""
    import dumbray_gb300 as dr

    table = {}
    best, best_ms, best_r = None, float("inf"), None
    total = batch.paths()
    for w in candidates:
        if w > 2 * max(total, 1):
            continue
        r = dr.Renderer(w, lanes)
        ms = _time_ms(lambda: batch.render(r, use_graph=use_graph), reps=1)
        table[w] = round(ms, 2)
        if ms < best_ms:
            if best_r is not None:
                best_r.close()
            best, best_ms, best_r = w, ms, r
        else:
            r.close()
    return best, table, best_r


def tune_block_shape(batch, renderer, shapes=(0, 1), use_graph=True):
    """Times one batch render with each traversal block shape on `renderer` (dr_renderer_set_block_shape);
    leaves the renderer on the fastest and returns (best, {shape: ms})."""
    table = {}
    for sh in shapes:
        renderer.set_block_shape(sh)
        table[sh] = round(_time_ms(lambda: batch.render(renderer, use_graph=use_graph), reps=1), 2)
    best = min(table, key=table.get)
    renderer.set_block_shape(best)
    return best, table


def representatives(jobs, n_tris):
    """The median-size job of every occupied size class: {class: job index}."""
    by = {}
    for i, n in enumerate(n_tris):
        by.setdefault(size_class(n), []).append(i)
    out = {}
    for cls, idx in by.items():
        idx = sorted(idx, key=lambda i: n_tris[i])
        out[cls] = idx[len(idx) // 2]
    return out
