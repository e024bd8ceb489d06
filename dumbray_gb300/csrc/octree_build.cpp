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

struct P3 {
    float x, y, z;
};
inline P3 mk(float x, float y, float z) { return P3{x, y, z}; }
inline P3 add(P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 scale(P3 a, float f) { return P3{a.x * f, a.y * f, a.z * f}; }
inline P3 divs(P3 a, float f) { float r = 1.0f / f; return P3{a.x * r, a.y * r, a.z * r}; }
inline P3 crs(P3 a, P3 v) { return P3{a.y * v.z - v.y * a.z, v.x * a.z - a.x * v.z, a.x * v.y - v.x * a.y}; }
inline float len(P3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline float comp(P3 v, int ax) { return ax == 0 ? v.x : (ax == 1 ? v.y : v.z); }

struct Bx {
    P3 lo, hi;
};
inline Bx fixed_box(P3 s, P3 e) {
    if (s.x > e.x) std::swap(s.x, e.x);
    if (s.y > e.y) std::swap(s.y, e.y);
    if (s.z > e.z) std::swap(s.z, e.z);
    return Bx{s, e};
}

struct T3 {
    P3 a, b, c;
};

// Vertex order by one axis (Triangle::sortByMases, Triangle.impl.h:183-196).
inline void order_by(T3 &t, int ax) {
    float am = comp(t.a, ax), bm = comp(t.b, ax), cm = comp(t.c, ax);
    if (am > bm) {
        if (cm > am) std::swap(t.a, t.b);
        else if (bm > cm) std::swap(t.a, t.c);
        else { P3 k = t.a; t.a = t.b; t.b = t.c; t.c = k; }
    } else {
        if (am > cm) { P3 k = t.a; t.a = t.c; t.c = t.b; t.b = k; }
        else if (bm > cm) std::swap(t.b, t.c);
    }
}
inline P3 lerp_at(P3 from, P3 to, float fv, float tv, float plane) { return add(from, scale(sub(to, from), (plane - fv) / (tv - fv))); }

// Piecewise slab clipping of one triangle against [s, e] on axis `ax`, emitting pieces through
// `emit`.  Returns early (true) as soon as `emit` returns true: the same routine serves the
// exact triangle/box overlap test (AABB::intersectsTri, AABB.impl.h:152-221, which recurses
// z -> x -> y and stops on the first surviving piece) and the clipping used for intersection
// centres and bounds (SHAPES_PUSH_INTERSECTIONS, Shapes.impl.cuh:178-262, which keeps all pieces).
template <class Emit>
bool slab_clip(T3 t, int ax, float s, float e, Emit &&emit) {
    order_by(t, ax);
    float av = comp(t.a, ax), bv = comp(t.b, ax), cv = comp(t.c, ax);
    if (cv < s || av > e) return false;
    if (av <= s) {
        P3 asc = lerp_at(t.a, t.c, av, cv, s);
        if (bv <= s) {
            P3 bsc = lerp_at(t.b, t.c, bv, cv, s);
            if (cv <= e) return emit(T3{asc, bsc, t.c});
            P3 bec = lerp_at(t.b, t.c, bv, cv, e);
            if (emit(T3{bsc, bec, asc})) return true;
            P3 aec = lerp_at(t.a, t.c, av, cv, e);
            return emit(T3{asc, bec, aec});
        }
        if (bv <= e) {
            if (cv <= e) {
                if (emit(T3{asc, t.b, t.c})) return true;
                P3 asb = lerp_at(t.a, t.b, av, bv, s);
                return emit(T3{asc, asb, t.b});
            }
            P3 asb = lerp_at(t.a, t.b, av, bv, s);
            P3 bec = lerp_at(t.b, t.c, bv, cv, e);
            if (emit(T3{asb, t.b, bec})) return true;
            if (emit(T3{asc, asb, bec})) return true;
            P3 aec = lerp_at(t.a, t.c, av, cv, e);
            return emit(T3{asc, bec, aec});
        }
        P3 asb = lerp_at(t.a, t.b, av, bv, s);
        P3 aeb = lerp_at(t.a, t.b, av, bv, e);
        if (emit(T3{asc, asb, aeb})) return true;
        P3 aec = lerp_at(t.a, t.c, av, cv, e);
        return emit(T3{asc, aeb, aec});
    }
    if (cv <= e) return emit(t);
    P3 aec = lerp_at(t.a, t.c, av, cv, e);
    if (bv <= e) {
        P3 bec = lerp_at(t.b, t.c, bv, cv, e);
        if (emit(T3{t.a, t.b, bec})) return true;
        return emit(T3{t.a, aec, bec});
    }
    P3 aeb = lerp_at(t.a, t.b, av, bv, e);
    return emit(T3{t.a, aeb, aec});
}

// Exact triangle/box overlap: axes z, then x, then y.
bool overlaps(const Bx &b, const T3 &t) {
    auto ylevel = [&](const T3 &p) { return slab_clip(p, 1, b.lo.y, b.hi.y, [](const T3 &) { return true; }); };
    auto xlevel = [&](const T3 &p) { return slab_clip(p, 0, b.lo.x, b.hi.x, ylevel); };
    return slab_clip(t, 2, b.lo.z, b.hi.z, xlevel);
}

// All pieces of t inside b (x, then y, then z), in the reference's order.
struct Pieces {
    T3 p[32];
    int n = 0;
};
void clip_all(const Bx &b, const T3 &t, Pieces &out) {
    Pieces x, y;
    slab_clip(t, 0, b.lo.x, b.hi.x, [&](const T3 &p) { if (x.n < 32) x.p[x.n++] = p; return false; });
    for (int i = 0; i < x.n; i++)
        slab_clip(x.p[i], 1, b.lo.y, b.hi.y, [&](const T3 &p) { if (y.n < 32) y.p[y.n++] = p; return false; });
    out.n = 0;
    for (int i = 0; i < y.n; i++)
        slab_clip(y.p[i], 2, b.lo.z, b.hi.z, [&](const T3 &p) { if (out.n < 32) out.p[out.n++] = p; return false; });
}

// Area-weighted centre of the clipped pieces (Shapes.impl.cuh:289-310).
P3 clipped_centre(const Bx &b, const T3 &t) {
    Pieces l;
    clip_all(b, t, l);
    if (l.n == 0) return divs(add(b.lo, b.hi), 2.0f);
    float total = 0.0f;
    P3 acc = mk(0, 0, 0);
    for (int i = 0; i < l.n; i++) {
        const T3 &p = l.p[i];
        float w = len(crs(sub(p.b, p.a), sub(p.c, p.a))) * 0.5f + 0.0001f;
        acc = add(acc, scale(divs(add(add(p.a, p.b), p.c), 3.0f), w));
        total += w;
    }
    return divs(acc, total);
}

// Bounds of the clipped pieces (Shapes.impl.cuh:265-287).
Bx clipped_bounds(const Bx &b, const T3 &t) {
    Pieces l;
    clip_all(b, t, l);
    if (l.n == 0) return b;
    P3 lo = b.hi, hi = b.lo;
    for (int i = 0; i < l.n; i++) {
        const T3 &p = l.p[i];
        const P3 v[3] = {p.a, p.b, p.c};
        for (int k = 0; k < 3; k++) {
            hi = mk(hi.x > v[k].x ? hi.x : v[k].x, hi.y > v[k].y ? hi.y : v[k].y, hi.z > v[k].z ? hi.z : v[k].z);
        }
        for (int k = 0; k < 3; k++) {
            lo = mk(lo.x < v[k].x ? lo.x : v[k].x, lo.y < v[k].y ? lo.y : v[k].y, lo.z < v[k].z ? lo.z : v[k].z);
        }
    }
    return fixed_box(lo, hi);
}

// The 8 overlapping octants around `c` (splitAABB, Octree.impl.cuh:423-434); child index
// bit 2 = upper x, bit 1 = upper y, bit 0 = upper z.
void octants(const Bx &b, P3 c, Bx *r, float E) {
    for (int i = 0; i < 8; i++) {
        P3 lo, hi;
        lo.x = (i & 4) ? c.x - E : b.lo.x;
        hi.x = (i & 4) ? b.hi.x : c.x + E;
        lo.y = (i & 2) ? c.y - E : b.lo.y;
        hi.y = (i & 2) ? b.hi.y : c.y + E;
        lo.z = (i & 1) ? c.z - E : b.lo.z;
        hi.z = (i & 1) ? b.hi.z : c.z + E;
        r[i] = fixed_box(lo, hi);
    }
}

// Shrink a node box to `lo..hi` padded by the octree epsilon, clamped to the old box
// (reduceNode tail, Octree.impl.cuh:526-532).
Bx shrink(const Bx &old, P3 lo, P3 hi, float E) {
    lo = sub(lo, mk(E, E, E));
    hi = add(hi, mk(E, E, E));
    lo = mk(std::fmax(lo.x, old.lo.x), std::fmax(lo.y, old.lo.y), std::fmax(lo.z, old.lo.z));
    hi = mk(std::fmin(hi.x, old.hi.x), std::fmin(hi.y, old.hi.y), std::fmin(hi.z, old.hi.z));
    return fixed_box(lo, hi);
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
        T3 t = tri((int32_t)i);
        P3 lo = mk(t.a.x < t.b.x ? t.a.x : t.b.x, t.a.y < t.b.y ? t.a.y : t.b.y, t.a.z < t.b.z ? t.a.z : t.b.z);
        lo = mk(lo.x < t.c.x ? lo.x : t.c.x, lo.y < t.c.y ? lo.y : t.c.y, lo.z < t.c.z ? lo.z : t.c.z);
        P3 hi = mk(t.a.x > t.b.x ? t.a.x : t.b.x, t.a.y > t.b.y ? t.a.y : t.b.y, t.a.z > t.b.z ? t.a.z : t.b.z);
        hi = mk(hi.x > t.c.x ? hi.x : t.c.x, hi.y > t.c.y ? hi.y : t.c.y, hi.z > t.c.z ? hi.z : t.c.z);
        Bx b = fixed_box(lo, hi);
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
