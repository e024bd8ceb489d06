"""Octree build on the GPU (dr_build_params.device_build = 1) against the host build: the same
tree bit for bit (node boxes, child links, leaf lists in order, root), on the reference's padding and
the physical-mode padding, from small edge cases up to the 1.31M-triangle displaced mesh."""
import time

import numpy as np
import pytest
import torch

import dumbray_gb300 as dr
from dumbray_gb300 import scenes

pytestmark = pytest.mark.gpu


def _same(tris, **kw):
    a = dr.build_octree_host(tris, **kw)
    b = dr.build_octree_host(tris, device_build=True, **kw)
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(np.asarray(x).view(np.int32), np.asarray(y).view(np.int32))
    return a[0]


@pytest.mark.parametrize("level", [1, 3, 5])
@pytest.mark.parametrize("eps", [0.0, dr.PHYSICAL_TREE])
def test_device_build_matches_host_build(cuda, level, eps):
    tris = np.concatenate([scenes.displaced_icosphere(level, 0.1, 1), scenes.box((3, 3, 3), inward=True)])
    _same(tris, box_epsilon=eps)


@pytest.mark.parametrize("n", [0, 1, 2, 7, 8, 9, 40])
def test_device_build_small_and_degenerate(cuda, n):
    rng = np.random.default_rng(n)
    tris = rng.uniform(-1, 1, (n, 3, 3)).astype(np.float32)
    if n >= 9:
        tris[3] = tris[2]                       # duplicate
        tris[4, 1] = tris[4, 0]                 # degenerate
    _same(tris)
    _same(tris, split_threshold=2, max_depth=6)


def test_device_build_full_mesh_and_scene(cuda):
    S = scenes.full_scene(8)
    t0 = time.time()
    st = _same(S["tris"], split_threshold=12, box_epsilon=dr.PHYSICAL_TREE)
    assert st["nodes"] > 100000
    # a scene built on the device casts like one built on the host
    a = dr.Scene(S["tris"], box_epsilon=dr.PHYSICAL_TREE, split_threshold=12)
    b = dr.Scene(S["tris"], box_epsilon=dr.PHYSICAL_TREE, split_threshold=12, device_build=True)
    o, d = scenes.incoherent_rays(20000, -1.1, 1.1, seed=5)
    to, td = torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda)
    ia, ta = dr.cast(a, to, td)
    ib, tb = dr.cast(b, to, td)
    assert torch.equal(ia, ib) and torch.equal(ta.view(torch.int32), tb.view(torch.int32))
    assert time.time() - t0 < 120
