"""The traversal's group-test boxes (dr_octree_group_planes), checked on the host.

The traversal tests the 8 children of a node group against a second copy of their boxes: the
reference's boxes with every empty leaf moved to a far point (gbox_ref, read by the counting
traversal of reference-padding scenes), and boxes refitted to the non-empty leaves below each child
(gbox, read by every other traversal).  A child may only be dropped if no leaf below it could accept
a hit, so these tests pin the two properties the hit- and count-preservation arguments rest on:
every refitted box is exactly the union of the non-empty leaf boxes below it (so it contains each of
them), and a ray that passes the reference's slab test (Shapes::castPreInversed<AABB>, the same
float32 operations as the kernels) of a non-empty leaf box also passes it for every refitted box on
the way down to that leaf."""
import numpy as np
import pytest

import dumbray_gb300 as dr
from dumbray_gb300 import scenes

FAR = np.float32(1e30)
K_EPS = np.float32(5e-6)   # VECTOR_EPSILON, the slab test's tolerance


def _scene():
    return np.concatenate([scenes.displaced_icosphere(3, 0.1, 2), scenes.box((3.0, 3.0, 3.0), inward=True),
                           scenes.quad((0.0, -1.4, 0.0), (6.0, 6.0), (0.0, 1.0, 0.0))])


def _planes_to_boxes(p):
    """[groups, 6, 8] planes -> [groups * 8, 6] boxes in export order 1 .."""
    return np.ascontiguousarray(p.transpose(0, 2, 1)).reshape(-1, 6)


def _refit(box, child, leaf):
    """Independent restatement: (live, lo, hi) per export node, bottom-up over the export order
    (children follow their parent)."""
    n = len(child)
    live = np.zeros(n, bool)
    lo = np.full((n, 3), np.inf, np.float32)
    hi = np.full((n, 3), -np.inf, np.float32)
    for i in range(n - 1, -1, -1):
        c = child[i]
        if c < 0:
            live[i] = leaf[i, 1] > 0
            if live[i]:
                lo[i], hi[i] = box[i, :3], box[i, 3:]
        else:
            kids = np.arange(c, c + 8)
            lk = kids[live[kids]]
            live[i] = len(lk) > 0
            if live[i]:
                lo[i] = lo[lk].min(0)
                hi[i] = hi[lk].max(0)
    return live, lo, hi


@pytest.mark.parametrize("padding", ["reference", "physical"])
def test_group_planes_match_their_definition(padding):
    tris = _scene()
    eps = 0.0 if padding == "reference" else dr.tight_box_epsilon(tris)
    box, child, leaf, g, r = dr.octree_group_planes_host(tris, split_threshold=4 if eps else 0, box_epsilon=eps)
    n = len(child)
    assert g.shape == ((n - 1) // 8, 6, 8) and r.shape == g.shape
    gb, rb = _planes_to_boxes(g), _planes_to_boxes(r)
    nodes = np.arange(1, n)
    empty = (child[nodes] < 0) & (leaf[nodes, 1] == 0)
    assert empty.any(), "the scene should have empty leaves"
    # gbox_ref: the reference's boxes, empty leaves at the far point
    assert np.array_equal(rb[~empty], box[nodes][~empty])
    assert np.all(rb[empty] == FAR)
    # gbox: exactly the union of the non-empty leaf boxes below, dead subtrees at the far point
    live, lo, hi = _refit(box, child, leaf)
    lv = live[nodes]
    assert np.array_equal(gb[lv, :3], lo[nodes][lv]) and np.array_equal(gb[lv, 3:], hi[nodes][lv])
    assert np.all(gb[~lv] == FAR)
    # refitted boxes never exceed the reference's
    assert np.all(gb[lv, :3] >= box[nodes][lv, :3]) and np.all(gb[lv, 3:] <= box[nodes][lv, 3:])
    # and they are smaller in total: the point of the refit
    def area(b):
        e = np.maximum(b[:, 3:] - b[:, :3], 0).astype(np.float64)
        return (e[:, 0] * e[:, 1] + e[:, 1] * e[:, 2] + e[:, 0] * e[:, 2]).sum()
    inner = child[nodes] >= 0
    assert area(gb[inner & lv]) < area(box[nodes][inner])


def _slab_pass(lo, hi, o, inv):
    """Shapes::castPreInversed<AABB>(clipBackface = false) in float32: per ray and box."""
    with np.errstate(invalid="ignore", over="ignore"):
        ds = (lo[None, :, :] - o[:, None, :]) * inv[:, None, :]
        de = (hi[None, :, :] - o[:, None, :]) * inv[:, None, :]
    mn = np.minimum(ds, de).max(axis=2)
    mx = np.maximum(ds, de).min(axis=2)
    return ~(mn > (mx + K_EPS)) & (mn != np.float32(np.finfo(np.float32).max))


@pytest.mark.parametrize("padding", ["reference", "physical"])
def test_refitted_boxes_keep_every_leaf_a_ray_reaches(padding):
    tris = _scene()
    eps = 0.0 if padding == "reference" else dr.tight_box_epsilon(tris)
    box, child, leaf, g, _ = dr.octree_group_planes_host(tris, split_threshold=4 if eps else 0, box_epsilon=eps)
    gb = _planes_to_boxes(g)
    n = len(child)
    parent = np.full(n, -1)
    for i in range(n):
        if child[i] >= 0:
            parent[child[i]:child[i] + 8] = i
    o, d = scenes.incoherent_rays(2000, -1.6, 1.6, seed=11)
    o = o.astype(np.float32)
    with np.errstate(divide="ignore"):
        inv = (np.float32(1.0) / d.astype(np.float32)).astype(np.float32)
    leaves = np.nonzero((child < 0) & (leaf[:, 1] > 0))[0]
    leaves = leaves[leaves > 0]
    rng = np.random.default_rng(3)
    leaves = rng.choice(leaves, size=min(400, len(leaves)), replace=False)
    hit_leaf = _slab_pass(box[leaves, :3], box[leaves, 3:], o, inv)       # [rays, leaves]
    checked = 0
    for k, e in enumerate(leaves):
        rays = np.nonzero(hit_leaf[:, k])[0]
        if len(rays) == 0:
            continue
        a = e
        while a > 0:   # the leaf itself and every ancestor below the root: their group-test boxes
            ok = _slab_pass(gb[a - 1, None, :3], gb[a - 1, None, 3:], o[rays], inv[rays])[:, 0]
            assert ok.all(), (padding, int(e), int(a))
            checked += int(ok.size)
            a = parent[a]
    assert checked > 1000


def test_group_planes_of_degenerate_trees():
    """A tree whose root is a leaf has no groups; a split tree whose triangles crowd into one corner
    keeps its other children as empty leaves at the far point in both plane sets."""
    one = scenes.quad((0.0, 0.0, 0.0), (1.0, 1.0), (0.0, 1.0, 0.0))
    box, child, leaf, g, r = dr.octree_group_planes_host(one)
    assert len(child) == 1 and g.shape[0] == 0 and r.shape[0] == 0
    # 400 small triangles near (0.75, 0.75, 0.75) and one at (-1, -1, -1): most octants stay empty
    rng = np.random.default_rng(5)
    c = rng.uniform(0.6, 0.9, size=(400, 1, 3)).astype(np.float32)
    small = c + rng.uniform(-0.01, 0.01, size=(400, 3, 3)).astype(np.float32)
    tris = np.concatenate([small, np.array([[[-1, -1, -1], [-0.99, -1, -1], [-1, -0.99, -1]]], np.float32)])
    box, child, leaf, g, r = dr.octree_group_planes_host(tris, split_threshold=4, box_epsilon=-1.0)
    gb, rb = _planes_to_boxes(g), _planes_to_boxes(r)
    nodes = np.arange(1, len(child))
    empty = (child[nodes] < 0) & (leaf[nodes, 1] == 0)
    assert empty.any()
    assert np.all(gb[empty] == FAR) and np.all(rb[empty] == FAR)
    live, lo, hi = _refit(box, child, leaf)
    assert live[0]
    lv = live[nodes]
    assert np.array_equal(gb[lv, :3], lo[nodes][lv]) and np.array_equal(gb[lv, 3:], hi[nodes][lv])
