// octree_build.cpp - host octree builder for the GB300 ray caster.
//
// Builds the same tree as DumbRay's Octree<Renderable<BakedTriFace>>::push + build
// (__source__/DataStructures/Objects/Scene/Raycasters/Octree/Octree.impl.cuh:97-129, 339-533),
// i.e. identical node boxes, split decisions and leaf triangle lists, but:
//   * level by level (breadth first) instead of recursively, so every level is one parallel pass
//     over all (node, triangle) references and the output is in BFS order;
//   * into flat arrays (no pointers): the 8 children of a node are consecutive and 8-aligned,
//     which is what the device traversal wants (one 256-byte group per inner node).
// The floating-point operation order of the reference is preserved (the expensive per-reference
// clipping runs in parallel, every order-sensitive float sum runs serially in list order), so the
// tree is bit-identical to the reference's on any thread count.  Compile with -ffp-contract=off.
#include "octree_build.h"
#include "octree_geom.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <functional>
#include <thread>

namespace drb {
namespace {

const float kEps = 0.000005f;               // VECTOR_EPSILON (Vector3.h:10)
const float kBoxEps = 0.000005f * 256.0f;   // OCTREE_AABB_EPSILON (Octree.impl.cuh:3-5)

using namespace geom;

// Host wrappers with their own scratch.
P3 clipped_centre(const Bx &b, const T3 &t) {
    Pieces l, x, y;
    return geom::clipped_centre(b, t, l, x, y);
}
Bx clipped_bounds(const Bx &b, const T3 &t) {
    Pieces l, x, y;
    return geom::clipped_bounds(b, t, l, x, y);
}

void parallel_for(int64_t n, int threads, const std::function<void(int64_t, int64_t)> &fn) {
    if (n <= 0) return;
    if (threads <= 1 || n < 2048) { fn(0, n); return; }
    const int64_t chunk = std::max<int64_t>(1024, n / (threads * 8));
    std::atomic<int64_t> next{0};
    auto work = [&]() {
        for (;;) {
            int64_t s = next.fetch_add(chunk);
            if (s >= n) break;
            fn(s, std::min(n, s + chunk));
        }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < threads; k++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
}

}  // namespace

bool build_octree(const float *xyz, int64_t n, const BuildOptions &opt, FlatOctree &out) {
    out = FlatOctree();
    if (n <= 0) return true;
    const int threads = opt.threads > 0 ? opt.threads : (int)std::max(1u, std::thread::hardware_concurrency());
    const int max_depth = opt.max_depth > 0 ? opt.max_depth : 24;
    const int split_n = opt.split_threshold > 0 ? opt.split_threshold : 8;
    float E = opt.box_eps > 0.0f ? opt.box_eps : kBoxEps;
    if (opt.box_eps < 0.0f) {  // scaled to the scene: 2^-18 x the largest absolute coordinate
        float m = 0.0f;
        for (int64_t i = 0; i < 9 * n; i++) m = std::fmax(m, std::fabs(xyz[i]));
        E = std::fmax(m, 1e-30f) * (1.0f / 262144.0f);
    }
    auto tri = [&](int32_t i) {
        const float *p = xyz + 9 * (int64_t)i;
        return T3{mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8])};
    };

    // Root box: union of triangle boxes padded by the octree epsilon, except that the first
    // triangle's box is taken unpadded (push, Octree.impl.cuh:97-111).
    Bx root;
    for (int64_t i = 0; i < n; i++) {
        Bx b = tri_box(tri((int32_t)i));
        if (i == 0) root = b;
        else {
            P3 bl = sub(b.lo, mk(E, E, E)), bh = add(b.hi, mk(E, E, E));
            root = fixed_box(mk(std::fmin(root.lo.x, bl.x), std::fmin(root.lo.y, bl.y), std::fmin(root.lo.z, bl.z)),
                             mk(std::fmax(root.hi.x, bh.x), std::fmax(root.hi.y, bh.y), std::fmax(root.hi.z, bh.z)));
        }
    }

    // Level state: nodes of the current level (BFS order) and their references, grouped per node
    // in the reference's list order.
    struct LevelNode {
        Bx box;
        int64_t ref_begin, ref_end;
        int64_t global;  // index in the final node array (-1 for the root)
    };
    std::vector<LevelNode> level{{root, 0, n, -1}};
    std::vector<int32_t> refs(n);
    for (int64_t i = 0; i < n; i++) refs[i] = (int32_t)i;

    // Final arrays.  Root stored separately; nodes[0..7] are the root's children.
    std::vector<Bx> boxes;
    std::vector<int32_t> child;     // first child index, or -1 for a leaf
    std::vector<int64_t> leaf_lo;   // leaf reference range
    std::vector<int32_t> leaf_cnt;
    std::vector<int32_t> leaf_refs;
    std::vector<int32_t> parent;    // for the bottom-up reduce
    std::vector<int32_t> depth_of;
    Bx root_box = root;
    int32_t root_child = -1;
    int64_t root_leaf_lo = 0;
    int32_t root_leaf_cnt = 0;
    int max_seen = 0;

    for (int depth = 0; !level.empty(); depth++) {
        max_seen = std::max(max_seen, depth);
        const int64_t nl = (int64_t)level.size();
        const int64_t nr = (int64_t)refs.size();
        // which level node owns each reference
        std::vector<int32_t> owner(nr);
        parallel_for(nl, threads, [&](int64_t s, int64_t e) {
            for (int64_t k = s; k < e; k++)
                for (int64_t r = level[k].ref_begin; r < level[k].ref_end; r++) owner[r] = (int32_t)k;
        });
        auto splittable = [&](int64_t k) {
            int64_t cnt = level[k].ref_end - level[k].ref_begin;
            return depth < max_depth && cnt >= split_n;
        };
        // (1) clipped centre of every reference of a splittable node, in parallel
        std::vector<P3> centre(nr);
        parallel_for(nr, threads, [&](int64_t s, int64_t e) {
            for (int64_t r = s; r < e; r++) {
                int64_t k = owner[r];
                if (splittable(k)) centre[r] = clipped_centre(level[k].box, tri(refs[r]));
            }
        });
        // (2) split point per node: serial float sum in list order
        std::vector<P3> split_at(nl);
        std::vector<std::array<Bx, 8>> sub(nl);
        parallel_for(nl, threads, [&](int64_t s, int64_t e) {
            for (int64_t k = s; k < e; k++) {
                if (!splittable(k)) continue;
                P3 c = mk(0, 0, 0);
                for (int64_t r = level[k].ref_begin; r < level[k].ref_end; r++) c = add(c, centre[r]);
                c = divs(c, (float)(level[k].ref_end - level[k].ref_begin));
                split_at[k] = c;
                octants(level[k].box, c, sub[k].data(), E);
            }
        });
        std::vector<P3>().swap(centre);
        // (3) octant overlap mask per reference
        std::vector<uint8_t> mask(nr, 0);
        parallel_for(nr, threads, [&](int64_t s, int64_t e) {
            for (int64_t r = s; r < e; r++) {
                int64_t k = owner[r];
                if (!splittable(k)) continue;
                T3 t = tri(refs[r]);
                uint8_t m = 0;
                for (int i = 0; i < 8; i++)
                    if (overlaps(sub[k][i], t)) m |= (uint8_t)(1u << i);
                mask[r] = m;
            }
        });
        // (4) split decision per node (splittingMakesSence, Octree.impl.cuh:437-475)
        std::vector<uint8_t> does_split(nl, 0);
        std::vector<std::array<int64_t, 8>> occupancy(nl);
        parallel_for(nl, threads, [&](int64_t s, int64_t e) {
            for (int64_t k = s; k < e; k++) {
                if (!splittable(k)) continue;
                int64_t cnt = level[k].ref_end - level[k].ref_begin;
                std::array<int64_t, 8> occ{};
                for (int64_t r = level[k].ref_begin; r < level[k].ref_end; r++)
                    for (int i = 0; i < 8; i++) occ[i] += (mask[r] >> i) & 1;
                int full = 0;
                float load = 0.0f;
                for (int i = 0; i < 8; i++) {
                    if (occ[i] >= cnt) full++;
                    load += ((float)occ[i]) / ((float)cnt);
                }
                bool ok = (full < 1) && (load < std::fmin(((float)cnt) / ((float)split_n), 6.0f));
                does_split[k] = ok ? 1 : 0;
                occupancy[k] = occ;
            }
        });
        // (5) leaves: shrink to the clipped content (reduceNode(index, true)) and emit their lists
        std::vector<Bx> leaf_box(nl);
        parallel_for(nl, threads, [&](int64_t s, int64_t e) {
            for (int64_t k = s; k < e; k++) {
                if (does_split[k]) continue;
                P3 lo = level[k].box.hi, hi = level[k].box.lo;
                for (int64_t r = level[k].ref_begin; r < level[k].ref_end; r++) {
                    Bx ob = clipped_bounds(level[k].box, tri(refs[r]));
                    lo = mk(std::fmin(lo.x, ob.lo.x), std::fmin(lo.y, ob.lo.y), std::fmin(lo.z, ob.lo.z));
                    hi = mk(std::fmax(hi.x, ob.hi.x), std::fmax(hi.y, ob.hi.y), std::fmax(hi.z, ob.hi.z));
                }
                leaf_box[k] = shrink(level[k].box, lo, hi, E);
            }
        });
        // (6) allocate the next level: children of splitting nodes, 8 consecutive, BFS order
        std::vector<LevelNode> next;
        std::vector<int64_t> child_ref_base;
        int64_t next_refs = 0;
        for (int64_t k = 0; k < nl; k++) {
            LevelNode &ln = level[k];
            if (!does_split[k]) {
                int64_t lo = (int64_t)leaf_refs.size();
                for (int64_t r = ln.ref_begin; r < ln.ref_end; r++) leaf_refs.push_back(refs[r]);
                int32_t cnt = (int32_t)(ln.ref_end - ln.ref_begin);
                if (ln.global < 0) { root_box = leaf_box[k]; root_leaf_lo = lo; root_leaf_cnt = cnt; }
                else { boxes[ln.global] = leaf_box[k]; leaf_lo[ln.global] = lo; leaf_cnt[ln.global] = cnt; }
                continue;
            }
            int64_t first = (int64_t)boxes.size();
            if (ln.global < 0) root_child = (int32_t)first;
            else child[ln.global] = (int32_t)first;
            for (int i = 0; i < 8; i++) {
                boxes.push_back(sub[k][i]);
                child.push_back(-1);
                leaf_lo.push_back(0);
                leaf_cnt.push_back(0);
                parent.push_back((int32_t)ln.global);
                depth_of.push_back(depth + 1);
                LevelNode c;
                c.box = sub[k][i];
                c.ref_begin = next_refs;
                next_refs += occupancy[k][i];
                c.ref_end = next_refs;
                c.global = first + i;
                next.push_back(c);
            }
        }
        // (7) child reference lists: for child i of node k, the parent's references whose mask has
        // bit i, in the parent's order (Octree.impl.cuh:392-404)
        std::vector<int32_t> next_list(next_refs);
        {
            std::vector<int64_t> first_child(nl, -1);
            int64_t c = 0;
            for (int64_t k = 0; k < nl; k++)
                if (does_split[k]) { first_child[k] = c; c += 8; }
            parallel_for(nl, threads, [&](int64_t s, int64_t e) {
                for (int64_t k = s; k < e; k++) {
                    if (first_child[k] < 0) continue;
                    for (int i = 0; i < 8; i++) {
                        int64_t w = next[first_child[k] + i].ref_begin;
                        for (int64_t r = level[k].ref_begin; r < level[k].ref_end; r++)
                            if ((mask[r] >> i) & 1) next_list[w++] = refs[r];
                    }
                }
            });
        }
        refs.swap(next_list);
        level.swap(next);
    }

    // Bottom-up reduce of inner nodes (reduceNode(0, false) after the build): each inner node
    // shrinks to the union of its children's boxes; deeper nodes first.
    const int64_t nn = (int64_t)boxes.size();
    std::vector<int64_t> order(nn);
    for (int64_t i = 0; i < nn; i++) order[i] = i;
    // BFS order has non-decreasing depth, so reverse index order is children-before-parents.
    for (int64_t i = nn - 1; i >= 0; i--) {
        if (child[i] < 0) continue;
        P3 lo = boxes[i].hi, hi = boxes[i].lo;
        for (int c = 0; c < 8; c++) {
            const Bx &cb = boxes[child[i] + c];
            lo = mk(std::fmin(lo.x, cb.lo.x), std::fmin(lo.y, cb.lo.y), std::fmin(lo.z, cb.lo.z));
            hi = mk(std::fmax(hi.x, cb.hi.x), std::fmax(hi.y, cb.hi.y), std::fmax(hi.z, cb.hi.z));
        }
        boxes[i] = shrink(boxes[i], lo, hi, E);
    }
    if (root_child >= 0) {
        P3 lo = root_box.hi, hi = root_box.lo;
        for (int c = 0; c < 8; c++) {
            const Bx &cb = boxes[root_child + c];
            lo = mk(std::fmin(lo.x, cb.lo.x), std::fmin(lo.y, cb.lo.y), std::fmin(lo.z, cb.lo.z));
            hi = mk(std::fmax(hi.x, cb.hi.x), std::fmax(hi.y, cb.hi.y), std::fmax(hi.z, cb.hi.z));
        }
        root_box = shrink(root_box, lo, hi, E);
    }

    out.node_count = nn;
    out.node_lo.resize(3 * nn);
    out.node_hi.resize(3 * nn);
    out.node_child = std::move(child);
    out.node_leaf_first.resize(nn);
    out.node_leaf_count = std::move(leaf_cnt);
    for (int64_t i = 0; i < nn; i++) {
        out.node_lo[3 * i] = boxes[i].lo.x; out.node_lo[3 * i + 1] = boxes[i].lo.y; out.node_lo[3 * i + 2] = boxes[i].lo.z;
        out.node_hi[3 * i] = boxes[i].hi.x; out.node_hi[3 * i + 1] = boxes[i].hi.y; out.node_hi[3 * i + 2] = boxes[i].hi.z;
        out.node_leaf_first[i] = leaf_lo[i];
    }
    out.root_lo[0] = root_box.lo.x; out.root_lo[1] = root_box.lo.y; out.root_lo[2] = root_box.lo.z;
    out.root_hi[0] = root_box.hi.x; out.root_hi[1] = root_box.hi.y; out.root_hi[2] = root_box.hi.z;
    out.root_child = root_child;
    out.root_leaf_first = root_leaf_lo;
    out.root_leaf_count = root_leaf_cnt;
    out.leaf_refs = std::move(leaf_refs);
    out.depth = max_seen;
    (void)parent;
    (void)depth_of;
    (void)kEps;
    return true;
}

}  // namespace drb
