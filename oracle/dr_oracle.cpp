// dr_oracle.cpp - CPU ORACLE for the DumbRay rendering hot path.  TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load this library, and
// only as the checker or the timed CPU baseline; the product (dumbray_gb300/) never links it.
//
// It restates, in plain single-file C++ (scalar float for the reference semantics, double for the
// physical-mode oracle), the algorithms of the reference's hot path.  Citations are
// file:line relative to the DumbRay checkout, __source__/ abbreviated S/:
//   octree build   S/DataStructures/Objects/Scene/Raycasters/Octree/Octree.impl.cuh:97-129,339-533
//   octree cast    Octree.impl.cuh:174-212 (traversal), :584-612 (castInLeaf)
//   triangle cast  S/DataStructures/Primitives/Compound/Triangle/Triangle.impl.h:283-348
//   slab test      S/DataStructures/Primitives/Compound/AABB/AABB.impl.h:116-130
//   tri/box clip   AABB.impl.h:152-221; S/Namespaces/Shapes/Shapes.impl.cuh:176-330
//   renderer       S/DataStructures/Renderers/DumbRenderer/DumbRenderer.cu:174-443
//   shaders        .../Shaders/DumbBasedShader/DumbBasedShader.impl.cuh:18-122,
//                  .../Shaders/SimpleStochasticShader/SimpleStochasticShader.impl.cuh:13-37
//   lights         .../Lights/SphericalLightEmitter/SphericalLightEmitter.impl.cuh:10-18,
//                  .../SimpleSoftDirectionalLight.impl.cuh:12-19, .../SimpleDirectionalLight.impl.cuh:13-16
//   lenses         .../Lenses/DefaultPerspectiveLense/DefaultPerspectiveLense.impl.cuh:5-19,
//                  .../SimpleStochasticLense.impl.cuh:4-25, .../SphericalSegmentLense.impl.cuh:6-36
//   frame buffer   S/DataStructures/Screen/FrameBuffer/BlockBasedFrameBuffer/BlockBasedFrameBuffer.impl.cuh:108-156
//
// Parity pin: the octree cast is checked hit-for-hit against the reference's own Octree::cast
// (compiled from the reference sources by oracle/build_ref.sh) and against committed golden
// vectors produced by that build (tests/golden/).  The reference renderer draws its random numbers
// from an XORWOW stream seeded by rand(), so per-sample agreement is impossible: the renderer
// restatement is pinned statistically (per-pixel RMSE at converged sample counts).
//
// Float arithmetic follows the reference's operation order exactly; build with -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <vector>
#include <thread>
#include <atomic>
#include <algorithm>
#include "../include/dr_api.h"

namespace {

const float EPS = 0.000005f;                 // VECTOR_EPSILON, Vector3.h:10
const float BOX_EPS = 0.000005f * 256.0f;    // OCTREE_AABB_EPSILON, Octree.impl.cuh:3-5
const float PI_F = 3.14159265359f;           // PI, Vector3.h:8
const float RADIAN_F = 57.29577951308233f;   // RADIAN, Vector3.h:9

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float f) { return V3{a.x * f, a.y * f, a.z * f}; }
// Vector3::operator/(float): multiplies by 1/f (Vector3.impl.h:175-178)
inline V3 divf(V3 a, float f) { float fi = 1.0f / f; return V3{a.x * fi, a.y * fi, a.z * fi}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// Vector3::operator& (Vector3.impl.h:19-22)
inline V3 cross(V3 a, V3 v) { return V3{a.y * v.z - v.y * a.z, v.x * a.z - a.x * v.z, a.x * v.y - v.x * a.y}; }
inline float sqrmag(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline float mag(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 normalized(V3 a) { float im = 1.0f / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); return V3{a.x * im, a.y * im, a.z * im}; }
inline bool veq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline V3 col3(const float *p) { return V3{p[0], p[1], p[2]}; }
inline V3 vmul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
// Vector3::reflection (Vector3.impl.h:418-421)
inline V3 reflection(V3 v, V3 n) { float m = (2.0f * dot(v, n) / sqrmag(n)); return V3{v.x - n.x * m, v.y - n.y * m, v.z - n.z * m}; }
// Vector3::normalOn: v * (dot(this, v) / |v|^2)
inline V3 normal_on(V3 a, V3 v) { return v * (dot(a, v) / sqrmag(v)); }

struct Box {
    V3 s, e;
};
// AABB(s, e) constructor with fix() (AABB.impl.h:11-15, 139-143)
inline Box mkbox(V3 s, V3 e) {
    if (s.x > e.x) std::swap(s.x, e.x);
    if (s.y > e.y) std::swap(s.y, e.y);
    if (s.z > e.z) std::swap(s.z, e.z);
    return Box{s, e};
}
inline bool contains(const Box &b, V3 v) {
    return v.x >= b.s.x && v.y >= b.s.y && v.z >= b.s.z && v.x <= b.e.x && v.y <= b.e.y && v.z <= b.e.z;
}

struct Tri {
    V3 a, b, c;
};

// Triangle::sortByMases (Triangle.impl.h:183-196)
inline void sort_by_masses(Tri &t, float am, float bm, float cm) {
    if (am > bm) {
        if (cm > am) std::swap(t.a, t.b);
        else {
            if (bm > cm) std::swap(t.a, t.c);
            else { V3 tmp = t.a; t.a = t.b; t.b = t.c; t.c = tmp; }
        }
    } else {
        if (am > cm) { V3 tmp = t.a; t.a = t.c; t.c = t.b; t.b = tmp; }
        else if (bm > cm) std::swap(t.b, t.c);
    }
}
inline float axis(V3 v, int ax) { return ax == 0 ? v.x : (ax == 1 ? v.y : v.z); }
inline void sort_axis(Tri &t, int ax) { sort_by_masses(t, axis(t.a, ax), axis(t.b, ax), axis(t.c, ax)); }
// CROSS_POINT (AABB.impl.h:149)
inline V3 cross_point(V3 from, V3 to, float fv, float tv, float barrier) { return from + (to - from) * ((barrier - fv) / (tv - fv)); }

// AABB::intersectsTri<dimm> (AABB.impl.h:128-221): dimm 0 -> z, 1 -> x, 2 -> y, 3 -> true.
bool intersects_tri(const Box &bx, Tri t, int dimm);
bool intersects_tri_range(const Box &bx, const Tri &t, float av, float bv, float cv, float s, float e, int dimm) {
    int nd = dimm + 1;
    if (cv < s) return false;
    if (av > e) return false;
    if (av <= s) {
        V3 asc = cross_point(t.a, t.c, av, cv, s);
        if (bv <= s) {
            V3 bsc = cross_point(t.b, t.c, bv, cv, s);
            if (cv <= e) return intersects_tri(bx, Tri{asc, bsc, t.c}, nd);
            V3 bec = cross_point(t.b, t.c, bv, cv, e);
            if (intersects_tri(bx, Tri{bsc, bec, asc}, nd)) return true;
            V3 aec = cross_point(t.a, t.c, av, cv, e);
            return intersects_tri(bx, Tri{asc, bec, aec}, nd);
        } else if (bv <= e) {
            if (cv <= e) {
                if (intersects_tri(bx, Tri{asc, t.b, t.c}, nd)) return true;
                V3 asb = cross_point(t.a, t.b, av, bv, s);
                return intersects_tri(bx, Tri{asc, asb, t.b}, nd);
            }
            V3 asb = cross_point(t.a, t.b, av, bv, s);
            V3 bec = cross_point(t.b, t.c, bv, cv, e);
            if (intersects_tri(bx, Tri{asb, t.b, bec}, nd)) return true;
            if (intersects_tri(bx, Tri{asc, asb, bec}, nd)) return true;
            V3 aec = cross_point(t.a, t.c, av, cv, e);
            return intersects_tri(bx, Tri{asc, bec, aec}, nd);
        } else {
            V3 asb = cross_point(t.a, t.b, av, bv, s);
            V3 aeb = cross_point(t.a, t.b, av, bv, e);
            if (intersects_tri(bx, Tri{asc, asb, aeb}, nd)) return true;
            V3 aec = cross_point(t.a, t.c, av, cv, e);
            return intersects_tri(bx, Tri{asc, aeb, aec}, nd);
        }
    } else {
        if (cv <= e) return intersects_tri(bx, t, nd);
        V3 aec = cross_point(t.a, t.c, av, cv, e);
        if (bv <= e) {
            V3 bec = cross_point(t.b, t.c, bv, cv, e);
            if (intersects_tri(bx, Tri{t.a, t.b, bec}, nd)) return true;
            return intersects_tri(bx, Tri{t.a, aec, bec}, nd);
        }
        V3 aeb = cross_point(t.a, t.b, av, bv, e);
        return intersects_tri(bx, Tri{t.a, aeb, aec}, nd);
    }
}
bool intersects_tri(const Box &bx, Tri t, int dimm) {
    if (dimm == 0) { sort_axis(t, 2); return intersects_tri_range(bx, t, t.a.z, t.b.z, t.c.z, bx.s.z, bx.e.z, 0); }
    if (dimm == 1) { sort_axis(t, 0); return intersects_tri_range(bx, t, t.a.x, t.b.x, t.c.x, bx.s.x, bx.e.x, 1); }
    if (dimm == 2) { sort_axis(t, 1); return intersects_tri_range(bx, t, t.a.y, t.b.y, t.c.y, bx.s.y, bx.e.y, 2); }
    return true;
}

// SHAPES_PUSH_INTERSECTIONS (Shapes.impl.cuh:178-262): clip every triangle of `front` to [s, e]
// along `ax`, appending the pieces to `back` in the reference's order.
struct TriList {
    Tri t[32];
    int n = 0;
    void push(const Tri &x) { if (n < 32) t[n++] = x; }
};
void clip_axis(TriList &front, TriList &back, int ax, float s, float e) {
    for (int i = 0; i < front.n; i++) {
        Tri &t = front.t[i];
        sort_axis(t, ax);
        float av = axis(t.a, ax), bv = axis(t.b, ax), cv = axis(t.c, ax);
        if (cv < s) continue;
        else if (av > e) continue;
        else if (av <= s) {
            V3 asc = cross_point(t.a, t.c, av, cv, s);
            if (bv <= s) {
                V3 bsc = cross_point(t.b, t.c, bv, cv, s);
                if (cv <= e) back.push(Tri{asc, bsc, t.c});
                else {
                    V3 bec = cross_point(t.b, t.c, bv, cv, e);
                    back.push(Tri{bsc, bec, asc});
                    V3 aec = cross_point(t.a, t.c, av, cv, e);
                    back.push(Tri{asc, bec, aec});
                }
            } else if (bv <= e) {
                if (cv <= e) {
                    back.push(Tri{asc, t.b, t.c});
                    V3 asb = cross_point(t.a, t.b, av, bv, s);
                    back.push(Tri{asc, asb, t.b});
                } else {
                    V3 asb = cross_point(t.a, t.b, av, bv, s);
                    V3 bec = cross_point(t.b, t.c, bv, cv, e);
                    back.push(Tri{asb, t.b, bec});
                    back.push(Tri{asc, asb, bec});
                    V3 aec = cross_point(t.a, t.c, av, cv, e);
                    back.push(Tri{asc, bec, aec});
                }
            } else {
                V3 asb = cross_point(t.a, t.b, av, bv, s);
                V3 aeb = cross_point(t.a, t.b, av, bv, e);
                back.push(Tri{asc, asb, aeb});
                V3 aec = cross_point(t.a, t.c, av, cv, e);
                back.push(Tri{asc, aeb, aec});
            }
        } else {
            if (cv <= e) back.push(t);
            else {
                V3 aec = cross_point(t.a, t.c, av, cv, e);
                if (bv <= e) {
                    V3 bec = cross_point(t.b, t.c, bv, cv, e);
                    back.push(Tri{t.a, t.b, bec});
                    back.push(Tri{t.a, aec, bec});
                } else {
                    V3 aeb = cross_point(t.a, t.b, av, bv, e);
                    back.push(Tri{t.a, aeb, aec});
                }
            }
        }
    }
    front.n = 0;
}
// SHAPES_GET_INTERSECTING_TRIANGLES: x, then y, then z.
void clip_to_box(const Box &bx, const Tri &t, TriList &out) {
    TriList tmp;
    tmp.push(t);
    out.n = 0;
    clip_axis(tmp, out, 0, bx.s.x, bx.e.x);
    clip_axis(out, tmp, 1, bx.s.y, bx.e.y);
    clip_axis(tmp, out, 2, bx.s.z, bx.e.z);
}
// intersectionCenter<AABB, Triangle> (Shapes.impl.cuh:289-310)
V3 intersection_center(const Box &bx, const Tri &t) {
    TriList l;
    clip_to_box(bx, t, l);
    if (l.n > 0) {
        float size = 0.0f;
        V3 sum = v3(0, 0, 0);
        for (int i = 0; i < l.n; i++) {
            const Tri &p = l.t[i];
            float surface = (mag(cross(p.b - p.a, p.c - p.a)) * 0.5f + 0.0001f);
            V3 mc = divf(p.a + p.b + p.c, 3.0f);
            sum = sum + mc * surface;
            size += surface;
        }
        return divf(sum, size);
    }
    return divf(bx.s + bx.e, 2.0f);
}
// intersectionBounds<AABB, Triangle> (Shapes.impl.cuh:265-287)
Box intersection_bounds(const Box &bx, const Tri &t) {
    TriList l;
    clip_to_box(bx, t, l);
    if (l.n == 0) return bx;
    V3 mn = bx.e, mx = bx.s;
#define SMAX(a, b) (((a) > (b)) ? (a) : (b))
#define SMIN(a, b) (((a) < (b)) ? (a) : (b))
    for (int i = 0; i < l.n; i++) {
        const Tri &p = l.t[i];
        mx = v3(SMAX(SMAX(SMAX(mx.x, p.a.x), p.b.x), p.c.x), SMAX(SMAX(SMAX(mx.y, p.a.y), p.b.y), p.c.y),
                SMAX(SMAX(SMAX(mx.z, p.a.z), p.b.z), p.c.z));
        mn = v3(SMIN(SMIN(SMIN(mn.x, p.a.x), p.b.x), p.c.x), SMIN(SMIN(SMIN(mn.y, p.a.y), p.b.y), p.c.y),
                SMIN(SMIN(SMIN(mn.z, p.a.z), p.b.z), p.c.z));
    }
    return mkbox(mn, mx);
}
// boundingBox<Triangle> (Shapes.impl.cuh:371-381)
Box tri_bounds(const Tri &t) {
    V3 s = v3(SMIN(SMIN(t.a.x, t.b.x), t.c.x), SMIN(SMIN(t.a.y, t.b.y), t.c.y), SMIN(SMIN(t.a.z, t.b.z), t.c.z));
    V3 e = v3(SMAX(SMAX(t.a.x, t.b.x), t.c.x), SMAX(SMAX(t.a.y, t.b.y), t.c.y), SMAX(SMAX(t.a.z, t.b.z), t.c.z));
    return mkbox(s, e);
}
#undef SMAX
#undef SMIN

// ------------------------------------------------------------------------------------------
// Octree (Octree.cuh:50-228)
struct Node {
    Box b;
    int child = -1;          // first of 8 consecutive children, -1 for a leaf
    std::vector<int> tris;   // leaf triangle list, in the reference's push order
};

struct Octree {
    std::vector<Tri> tri;
    std::vector<Node> nodes;
    int max_depth = 24, split_n = 8;
    std::atomic<int> lock_flag{0};

    // splitAABB (Octree.impl.cuh:423-434)
    static void split_box(const Box &b, V3 c, Box *r) {
        V3 s = b.s, e = b.e;
        const float E = BOX_EPS;
        V3 ev = v3(E, E, E);
        r[0] = mkbox(s, c + ev);
        r[1] = mkbox(v3(s.x, s.y, c.z - E), v3(c.x + E, c.y + E, e.z));
        r[2] = mkbox(v3(s.x, c.y - E, s.z), v3(c.x + E, e.y, c.z + E));
        r[3] = mkbox(v3(s.x, c.y - E, c.z - E), v3(c.x + E, e.y, e.z));
        r[4] = mkbox(v3(c.x - E, s.y, s.z), v3(e.x, c.y + E, c.z + E));
        r[5] = mkbox(v3(c.x - E, s.y, c.z - E), v3(e.x, c.y + E, e.z));
        r[6] = mkbox(v3(c.x - E, c.y - E, s.z), v3(e.x, e.y, c.z + E));
        r[7] = mkbox(c - ev, e);
    }

    // reduceNode for a leaf (Octree.impl.cuh:489-533, reduceLeaves = true)
    static void reduce_leaf(Node &nd, const std::vector<Tri> &tri) {
        V3 st = nd.b.e, en = nd.b.s;
        for (int id : nd.tris) {
            Box ob = intersection_bounds(nd.b, tri[id]);
            st = v3(std::fmin(st.x, ob.s.x), std::fmin(st.y, ob.s.y), std::fmin(st.z, ob.s.z));
            en = v3(std::fmax(en.x, ob.e.x), std::fmax(en.y, ob.e.y), std::fmax(en.z, ob.e.z));
        }
        finish_reduce(nd, st, en);
    }
    static void finish_reduce(Node &nd, V3 st, V3 en) {
        V3 ev = v3(BOX_EPS, BOX_EPS, BOX_EPS);
        st = st - ev;
        en = en + ev;
        V3 bs = nd.b.s, be = nd.b.e;
        st = v3(std::fmax(st.x, bs.x), std::fmax(st.y, bs.y), std::fmax(st.z, bs.z));
        en = v3(std::fmin(en.x, be.x), std::fmin(en.y, be.y), std::fmin(en.z, be.z));
        nd.b = mkbox(st, en);
    }

    // split (Octree.impl.cuh:339-421) on a private subtree vector; returns the subtree rooted at
    // `root` as a list of nodes (index 0 = root) so subtrees can be built on different threads.
    void split_rec(std::vector<Node> &out, int idx, int depth) {
        Node &nd0 = out[idx];
        int count = (int)nd0.tris.size();
        if (depth >= max_depth || count < split_n) { reduce_leaf(out[idx], tri); return; }
        V3 center = v3(0, 0, 0);
        for (int id : nd0.tris) center = center + intersection_center(nd0.b, tri[id]);
        center = divf(center, (float)count);
        Box sub[8];
        split_box(nd0.b, center, sub);
        // splittingMakesSence (Octree.impl.cuh:437-475)
        std::vector<uint8_t> cache(count, 0);
        int full = 0;
        float load = 0.0f;
        for (int i = 0; i < 8; i++) {
            int ins = 0;
            for (int j = 0; j < count; j++)
                if (intersects_tri(sub[i], tri[out[idx].tris[j]], 0)) { ins++; cache[j] |= (uint8_t)(1 << i); }
            if (ins >= count) full++;
            load += ((float)ins) / ((float)count);
        }
        bool ok = (full < 1) && (load < std::fmin(((float)count) / ((float)split_n), 6.0f));
        if (!ok) { reduce_leaf(out[idx], tri); return; }
        int first = (int)out.size();
        out.resize(out.size() + 8);
        Node &nd = out[idx];
        nd.child = first;
        for (int i = 0; i < 8; i++) out[first + i].b = sub[i];
        for (int j = 0; j < count; j++)
            for (int i = 0; i < 8; i++)
                if (cache[j] & (1 << i)) out[first + i].tris.push_back(nd.tris[j]);
        std::vector<int>().swap(out[idx].tris);
        for (int i = 0; i < 8; i++) split_rec(out, first + i, depth + 1);
    }

    // reduceNode(0, false) after the build (Octree.impl.cuh:122-128, 489-533): inner nodes shrink
    // to the union of their children; leaves stay as reduced during the split.
    void reduce_inner(int idx) {
        Node &nd = nodes[idx];
        if (nd.child < 0) return;
        for (int i = 0; i < 8; i++) reduce_inner(nd.child + i);
        V3 st = nd.b.e, en = nd.b.s;
        for (int i = 0; i < 8; i++) {
            const Box &cb = nodes[nd.child + i].b;
            st = v3(std::fmin(st.x, cb.s.x), std::fmin(st.y, cb.s.y), std::fmin(st.z, cb.s.z));
            en = v3(std::fmax(en.x, cb.e.x), std::fmax(en.y, cb.e.y), std::fmax(en.z, cb.e.z));
        }
        finish_reduce(nodes[idx], st, en);
    }

    void build(int threads) {
        nodes.clear();
        nodes.emplace_back();
        // push (Octree.impl.cuh:97-111): root box grows by each triangle's box +- BOX_EPS,
        // except the first triangle, whose box is taken as is.
        V3 ev = v3(BOX_EPS, BOX_EPS, BOX_EPS);
        for (size_t i = 0; i < tri.size(); i++) {
            Box b = tri_bounds(tri[i]);
            if (i == 0) nodes[0].b = b;
            else {
                V3 os = nodes[0].b.s, oe = nodes[0].b.e;
                V3 bs = b.s - ev, be = b.e + ev;
                nodes[0].b = mkbox(v3(std::fmin(os.x, bs.x), std::fmin(os.y, bs.y), std::fmin(os.z, bs.z)),
                                   v3(std::fmax(oe.x, be.x), std::fmax(oe.y, be.y), std::fmax(oe.z, be.z)));
            }
            nodes[0].tris.push_back((int)i);
        }
        if (tri.empty()) return;
        // Split the top two levels serially, then finish every level-2 subtree on its own thread.
        std::vector<Node> top;
        top.push_back(std::move(nodes[0]));
        nodes.clear();
        top_split(top, 0, 0, 2);
        std::vector<int> pending;
        for (size_t i = 0; i < top.size(); i++)
            if (top[i].child == -1 && top_open[i]) pending.push_back((int)i);
        std::vector<std::vector<Node>> sub(pending.size());
        std::atomic<size_t> next{0};
        if (threads < 1) threads = 1;
        auto work = [&]() {
            for (;;) {
                size_t k = next.fetch_add(1);
                if (k >= pending.size()) break;
                sub[k].push_back(std::move(top[pending[k]]));
                split_rec(sub[k], 0, top_depth_of(pending[k]));
            }
        };
        std::vector<std::thread> pool;
        for (int k = 1; k < threads; k++) pool.emplace_back(work);
        work();
        for (auto &t : pool) t.join();
        // splice subtrees back, renumbering child links
        nodes = std::move(top);
        for (size_t k = 0; k < pending.size(); k++) {
            int base = (int)nodes.size();
            int at = pending[k];
            std::vector<Node> &s = sub[k];
            for (size_t j = 1; j < s.size(); j++) {
                Node nd = std::move(s[j]);
                if (nd.child >= 0) nd.child = nd.child - 1 + base;
                nodes.push_back(std::move(nd));
            }
            Node r = std::move(s[0]);
            if (r.child >= 0) r.child = r.child - 1 + base;
            nodes[at] = std::move(r);
        }
        reduce_inner(0);
    }

    // top-level split bookkeeping: depth per node and which leaves still need splitting
    std::vector<int> top_depth;
    std::vector<uint8_t> top_open;
    void top_split(std::vector<Node> &out, int idx, int depth, int stop) {
        if ((int)top_depth.size() < (int)out.size()) { top_depth.resize(out.size(), 0); top_open.resize(out.size(), 0); }
        top_depth[idx] = depth;
        if (depth >= stop) {
            top_open[idx] = 1;
            return;
        }
        size_t before = out.size();
        split_one(out, idx, depth);
        if (out.size() > before) {
            top_depth.resize(out.size(), 0);
            top_open.resize(out.size(), 0);
            int first = out[idx].child;
            for (int i = 0; i < 8; i++) top_split(out, first + i, depth + 1, stop);
        }
    }
    bool need_split_mark(const Node &) { return true; }
    int top_depth_of(int idx) { return top_depth[idx]; }
    // One split step (no recursion): either turns out[idx] into a reduced leaf or gives it 8 children.
    void split_one(std::vector<Node> &out, int idx, int depth) {
        int count = (int)out[idx].tris.size();
        if (depth >= max_depth || count < split_n) { reduce_leaf(out[idx], tri); out[idx].child = -2; return; }
        V3 center = v3(0, 0, 0);
        for (int id : out[idx].tris) center = center + intersection_center(out[idx].b, tri[id]);
        center = divf(center, (float)count);
        Box sub[8];
        split_box(out[idx].b, center, sub);
        std::vector<uint8_t> cache(count, 0);
        int full = 0;
        float load = 0.0f;
        for (int i = 0; i < 8; i++) {
            int ins = 0;
            for (int j = 0; j < count; j++)
                if (intersects_tri(sub[i], tri[out[idx].tris[j]], 0)) { ins++; cache[j] |= (uint8_t)(1 << i); }
            if (ins >= count) full++;
            load += ((float)ins) / ((float)count);
        }
        bool ok = (full < 1) && (load < std::fmin(((float)count) / ((float)split_n), 6.0f));
        if (!ok) { reduce_leaf(out[idx], tri); out[idx].child = -2; return; }
        int first = (int)out.size();
        out.resize(out.size() + 8);
        out[idx].child = first;
        for (int i = 0; i < 8; i++) out[first + i].b = sub[i];
        for (int j = 0; j < count; j++)
            for (int i = 0; i < 8; i++)
                if (cache[j] & (1 << i)) out[first + i].tris.push_back(out[idx].tris[j]);
        std::vector<int>().swap(out[idx].tris);
    }

    // AABB::castPreInversed + Shapes::castPreInversed<AABB>(.., false) (AABB.impl.h:116-130,
    // Shapes.impl.cuh:143-147)
    static bool slab(const Box &b, V3 o, V3 inv) {
        float ds = (b.s.x - o.x) * inv.x;
        float de = (b.e.x - o.x) * inv.x;
        float mn = std::fmin(ds, de), mx = std::fmax(ds, de);
        ds = (b.s.y - o.y) * inv.y;
        de = (b.e.y - o.y) * inv.y;
        mn = std::fmax(mn, std::fmin(ds, de));
        mx = std::fmin(mx, std::fmax(ds, de));
        ds = (b.s.z - o.z) * inv.z;
        de = (b.e.z - o.z) * inv.z;
        mn = std::fmax(mn, std::fmin(ds, de));
        mx = std::fmin(mx, std::fmax(ds, de));
        if (mn > mx + EPS) return false;
        return mn != FLT_MAX;
    }

    // Triangle::containsVertex (Triangle.impl.h:283-302)
    static bool contains_vertex(const Tri &t, V3 p) {
        if (veq(t.a, t.b) || veq(t.b, t.c) || veq(t.c, t.a)) return false;
        if (veq(p, t.a) || veq(p, t.b) || veq(p, t.c)) return true;
        V3 ab = t.b - t.a, bc = t.c - t.b, ca = t.a - t.c;
        V3 ax = p - t.a, bx = p - t.b, cx = p - t.c;
        const float S = 32 * EPS;
        return (dot(ab, ax) / mag(ax) + S >= -dot(ab, ca) / mag(ca)) &&
               (dot(bc, bx) / mag(bx) + S >= -dot(bc, ab) / mag(ab)) &&
               (dot(ca, cx) / mag(cx) + S >= -dot(ca, bc) / mag(bc));
    }
    // Triangle::cast (Triangle.impl.h:334-348)
    static bool tri_cast(const Tri &t, V3 o, V3 d, bool clip, float &dist, V3 &hp) {
        V3 n = cross(t.b - t.a, t.c - t.a);
        float dp = dot(t.a - o, n);
        if (clip && (dp < -EPS)) return false;
        float dirp = dot(d, n);
        if (dp * dirp <= 0) return false;
        float distance = dp / dirp;
        V3 hv = o + d * distance;
        if (contains_vertex(t, hv)) { dist = distance; hp = hv; return true; }
        return false;
    }

    // Octree::cast (Octree.impl.cuh:174-212) with castInLeaf (:584-612); `ignore` plays the
    // validateNotSameAsObject validator.  Counts child-box slab tests and triangle tests.
    int cast(V3 o, V3 d, bool clip, int ignore, float &t_out, V3 &p_out, long long *boxes, long long *tests) const {
        if (nodes.empty()) return -1;
        V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        if (nodes[0].child < 0) return cast_leaf(0, o, d, clip, ignore, t_out, p_out, tests);
        if (boxes) (*boxes)++;
        if (!slab(nodes[0].b, o, inv)) return -1;
        int order = (d.z < 0 ? 1 : 0) + (d.y < 0 ? 2 : 0) + (d.x < 0 ? 4 : 0);
        int st_node[32];
        int st_cur[32];
        int sp = 0;
        st_node[0] = nodes[0].child;
        st_cur[0] = 0;
        for (;;) {
            int child = -1;
            while (st_cur[sp] < 8) {
                int c = st_node[sp] + (order ^ st_cur[sp]);
                if (boxes) (*boxes)++;
                if (slab(nodes[c].b, o, inv)) { child = c; break; }
                st_cur[sp]++;
            }
            if (st_cur[sp] >= 8) {
                if (sp == 0) return -1;
                sp--;
            } else {
                if (nodes[child].child < 0) {
                    int h = cast_leaf(child, o, d, clip, ignore, t_out, p_out, tests);
                    if (h >= 0) return h;
                } else {
                    sp++;
                    st_node[sp] = nodes[child].child;
                    st_cur[sp] = 0;
                }
                st_cur[sp - ((nodes[child].child < 0) ? 0 : 1)]++;
            }
        }
    }
    int cast_leaf(int idx, V3 o, V3 d, bool clip, int ignore, float &t_out, V3 &p_out, long long *tests) const {
        const Node &nd = nodes[idx];
        if (nd.tris.empty()) return -1;
        float best = FLT_MAX;
        V3 bp = v3(0, 0, 0);
        int bi = -1;
        for (int id : nd.tris) {
            float dist;
            V3 hp;
            if (tests) (*tests)++;
            bool c = tri_cast(tri[id], o, d, clip, dist, hp);
            if (c && id == ignore) c = false;
            if (c && dist < best) { best = dist; bp = hp; bi = id; }
        }
        if (best != FLT_MAX && contains(nd.b, bp)) { t_out = best; p_out = bp; return bi; }
        return -1;
    }
};

// ------------------------------------------------------------------------------------------
// Counter-based random numbers: u32 = H(H(key + GOLDEN * (bounce * 128 + dim + 1))), where
// key = H(H(H(seed ^ 0x2545F491) ^ pixel) + sample) and H is the `lowbias32` integer hash
// (C. Wellons' public-domain hash-prospector result).  Float = (u >> 8) * 2^-24 in [0, 1).
inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16; return x;
}
inline uint32_t path_key(uint32_t seed, uint32_t pixel, uint32_t sample) {
    return hash32(hash32(hash32(seed ^ 0x2545F491U) ^ pixel) + sample);
}
inline float rnd(uint32_t key, uint32_t bounce, uint32_t dim) {
    uint32_t u = hash32(hash32(key + 0x9E3779B9U * (bounce * 128U + dim + 1U)));
    return (float)(u >> 8) * (1.0f / 16777216.0f);
}
inline double rndd(uint32_t key, uint32_t bounce, uint32_t dim) { return (double)rnd(key, bounce, dim); }
const uint32_t LENS_BOUNCE = 1023;

// DumbRand::pointOnSphere (DumbRand.impl.cuh:70-77) from two given uniforms
inline V3 point_on_sphere(float u0, float u1, float radius) {
    float theta = (2.0f * 3.14159265359f * u0);
    float cosPhi = (1.0f - (2.0f * u1));
    float sinPhi = std::sqrt(1.0f - (cosPhi * cosPhi));
    return v3((sinPhi * std::cos(theta)) * radius, (sinPhi * std::sin(theta)) * radius, cosPhi * radius);
}

// Triangle::getMasses (Triangle.impl.h:248-276)
V3 get_masses(const Tri &t, V3 center) {
    V3 ab = t.b - t.a;
    V3 bc = t.c - t.b;
    V3 ae = ab - normal_on(ab, bc);
    V3 ax = center - t.a;
    V3 ad = normal_on(ax, ae);
    if (ae.x < 0) { ad.x = -ad.x; ae.x = -ae.x; }
    if (ae.y < 0) { ad.y = -ad.y; ae.y = -ae.y; }
    if (ae.z < 0) { ad.z = -ad.z; ae.z = -ae.z; }
    float div = ad.x + ad.y + ad.z;
    if (div == 0) return v3(1, 0, 0);
    float g = (ae.x + ae.y + ae.z) / div;
    float tt;
    V3 by = t.a + ax * g - t.b;
    if (bc.x < 0) { bc.x = -bc.x; by.x = -by.x; }
    if (bc.y < 0) { bc.y = -bc.y; by.y = -by.y; }
    if (bc.z < 0) { bc.z = -bc.z; by.z = -by.z; }
    div = bc.x + bc.y + bc.z;
    if (div == 0) tt = 0;
    else tt = (by.x + by.y + by.z) / div;
    float cc = tt, bb = (1 - tt), aa = (g - 1);
    return divf(v3(aa, bb, cc), aa + bb + cc);
}
inline V3 mass_center(const Tri &t, V3 m) { return t.a * m.x + t.b * m.y + t.c * m.z; }
// Triangle::normal() = (c - a) x (b - a) (Triangle.impl.h:233-235)
inline V3 tri_normal(const Tri &t) { return cross(t.c - t.a, t.b - t.a); }

struct Col {
    float r, g, b;
};
inline Col operator+(Col a, Col b) { return Col{a.r + b.r, a.g + b.g, a.b + b.b}; }
inline Col operator*(Col a, Col b) { return Col{a.r * b.r, a.g * b.g, a.b * b.b}; }
inline Col operator*(Col a, float f) { return Col{a.r * f, a.g * f, a.b * f}; }
inline Col col(const float *p) { return Col{p[0], p[1], p[2]}; }
inline float clamp01(float v) { return std::fmax(0.0f, std::fmin(v, 1.0f)); }

// Lights::Spotlight constructor state (Spotlight.impl.cuh:5-33).
struct Spot {
    Col color;  // colour x luminosity
    V3 direction;
    float emitter, inner_cos, outer_cos, falloff;
    int samples;
    bool shadows, sphere;
};
Spot spot_state(const dr_light &l) {
    Spot s;
    s.color = Col{l.color[0] * l.luminosity, l.color[1] * l.luminosity, l.color[2] * l.luminosity};
    s.direction = normalized(col3(l.direction));
    s.emitter = (l.emitter_size < (32 * EPS)) ? (32 * EPS) : l.emitter_size;
    float inner = l.hotspot_angle, outer = l.falloff_angle;
    if (inner < 0.0f) inner = (-inner);
    if (inner > 180.0f) inner = 180.0f;
    if (outer < 0.0f) outer = (-inner);
    if (outer > 180.0f) outer = 180.0f;
    if (outer < inner) outer = inner;
    s.inner_cos = std::cos(inner * PI_F / 180.0f);
    s.outer_cos = std::cos(outer * PI_F / 180.0f);
    s.falloff = l.falloff_power;
    s.samples = (l.samples > 0) ? ((l.samples > 16) ? 16 : l.samples) : 0;
    s.shadows = l.cast_shadows != 0;
    s.sphere = l.emit_from_sphere != 0;
    return s;
}

struct Scene {
    Octree tree;
    std::vector<Tri> nrm;
    std::vector<int> mat;
    std::vector<dr_material> mats;
    std::vector<dr_light> lights;
    std::vector<struct Spot> spots;                // per light; spotlight constructor state
    struct Tex {
        int w, h, filter;
        std::vector<float> rgba;  // [h][w][4]
    };
    std::vector<Tex> tex;                          // dro_scene_set_textures
    std::vector<float> uv;                         // [n][3][2] corner texture coordinates
    std::vector<float> albedo, emission, rough;  // physical-mode per-triangle params
    std::vector<int> emissive;                   // emissive triangle ids
    std::vector<double> emissive_cdf;            // by power (luminance-free: r+g+b) x area
    double emissive_total = 0.0;
    // dro_scene_freeze_sampling: per-triangle power used for light selection and its pdfs, fixed at
    // the time of the call (the device library's sampling tables stay fixed when parameters are
    // written in place); empty = follow the current emission
    std::vector<double> frozen_power;
};

// ---- textures (Texture.impl.cuh:81-95; ColoredTexture, DumbStructs.cuh:88-131) ------------------
struct F4 {
    float x, y, z, w;
};
inline F4 f4add(F4 a, F4 b) { return F4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline F4 f4mul(F4 a, float f) { return F4{a.x * f, a.y * f, a.z * f, a.w * f}; }
inline F4 texel(const Scene::Tex &t, uint32_t x, uint32_t y) {
    const float *p = &t.rgba[4 * ((size_t)y * (size_t)t.w + x)];
    return F4{p[0], p[1], p[2], p[3]};
}
F4 tex_lookup(const Scene &S, int ti, float u, float v) {
    const Scene::Tex &t = S.tex[(size_t)ti];
    const uint32_t w = (uint32_t)t.w, h = (uint32_t)t.h;
    float x = (u + ((float)(((int)(-u)) + 2)));
    x -= ((float)((int)x));
    float y = (v + ((float)(((int)(-v)) + 2)));
    y -= ((float)((int)y));
    y = (1.0f - y);
    const float px = (x * ((float)w)), py = (y * ((float)h));
    const uint32_t min_x = (((uint32_t)px) % w), min_y = (((uint32_t)py) % h);
    const uint32_t max_x = ((min_x + 1) % w), max_y = ((min_y + 1) % h);
    const float off_x = (px - ((float)min_x)), off_y = (py - ((float)min_y));
    if (t.filter == DR_FILTER_NONE) return texel(t, (off_x <= 0.5f) ? min_x : max_x, (off_y <= 0.5f) ? min_y : max_y);
    return f4add(f4add(f4add(f4mul(texel(t, min_x, min_y), ((1.0f - off_x) * (1.0f - off_y))),
                             f4mul(texel(t, min_x, max_y), ((1.0f - off_x) * off_y))),
                       f4mul(texel(t, max_x, min_y), (off_x * (1.0f - off_y)))),
                 f4mul(texel(t, max_x, max_y), (off_x * off_y)));
}
struct UV {
    float u, v;
};
UV hit_uv(const Scene &S, int tri, V3 m) {
    const float *p = &S.uv[6 * (size_t)tri];
    return UV{((p[0] * m.x) + (p[2] * m.y)) + (p[4] * m.z), ((p[1] * m.x) + (p[3] * m.y)) + (p[5] * m.z)};
}
bool any_texture(const dr_material &m) { return m.texture[0] > 0 || m.texture[1] > 0 || m.texture[2] > 0 || m.texture[3] > 0; }
F4 channel_texel(const Scene &S, const dr_material &m, int ch, UV uv) {
    return tex_lookup(S, m.texture[ch] - 1, (uv.u * m.tiling[ch][0]) + m.offset[ch][0], (uv.v * m.tiling[ch][1]) + m.offset[ch][1]);
}
bool cut_out(const Scene &S, const dr_material &m, UV uv) {
    return m.texture[DR_TEX_ALPHA] > 0 && m.alpha_threshold >= (1.0f * channel_texel(S, m, DR_TEX_ALPHA, uv).w);
}
// ColoredTexture::getNormal (DumbStructs.cuh:99-131): the interpolated normal, or the normal map in
// the frame of that normal, a tangent from the corner texture coordinates and their cross product.
V3 shading_normal(const Scene &S, const dr_material &m, int tri, const Tri &v, const Tri &nt, V3 masses, UV uv) {
    V3 n = normalized(mass_center(nt, masses));
    if (m.texture[DR_TEX_NORMAL] <= 0) return n;
    const float *p = &S.uv[6 * (size_t)tri];
    UV td;
    V3 vd;
    const V3 mc = mass_center(v, masses);
    if (masses.x < 0.999f) {
        td = UV{p[0] - uv.u, p[1] - uv.v};
        vd = v.a - mc;
    } else {
        td = UV{p[2] - uv.u, p[3] - uv.v};
        vd = v.b - mc;
    }
    const V3 co = normalized(cross(vd, n));
    vd = cross(co, n);
    const V3 u = normalized((vd * td.v) - (co * td.u));
    const V3 w = cross(u, n);
    const F4 rgb = channel_texel(S, m, DR_TEX_NORMAL, uv);
    const V3 k = v3(m.normal_color[1] * rgb.z, m.normal_color[0] * ((rgb.x * 2.0f) - 1.0f), m.normal_color[2] * ((rgb.y * 2.0f) - 1.0f));
    return normalized(((n * k.x) + (u * k.y)) + (w * k.z));
}

// DumbBasedShader::requestIndirectSamples (DumbBasedShader.impl.cuh:18-62).  Returns false when no
// sample is produced (specular branch with n.ray >= 0); `type` gets the sample type (1 or 2).
bool dumb_based_request(const Scene &S, int tri, const dr_material &m, const Tri &v, const Tri &nt, V3 hit, V3 raydir,
                        uint32_t key, uint32_t bounce, V3 &dir, int &type) {
    V3 normal = normalized(tri_normal(v));
    V3 masses = get_masses(v, hit);
    const bool textured = any_texture(m);
    const UV uv = textured ? hit_uv(S, tri, masses) : UV{0.0f, 0.0f};
    if (textured && cut_out(S, m, uv)) {
        dir = raydir;
        type = 3;
        return true;
    }
    float metal = std::fmax(std::fmin(m.metal, 1.0f), 0.0f);
    if (rnd(key, bounce, 0) <= metal) {
        V3 n = shading_normal(S, m, tri, v, nt, masses, uv);
        if (dot(n, raydir) >= 0.0f) return false;
        V3 r = normalized(reflection(raydir, n));
        if (dot(r, normal) < 0) normal = normal * -1.0f;
        V3 a = cross(r, v3(1.0f, 0.0f, 0.0f));
        if (sqrmag(normal) < EPS) a = cross(r, v3(0.0f, 1.0f, 0.0f));
        a = normalized(a);
        V3 b = cross(r, a);
        V3 sd = v3(0, 0, 0);
        for (int tries = 0; tries < 32; tries++) {
            float cosine = std::pow(rnd(key, bounce, 8 + 2 * tries), 1.0f / m.specular);
            float sinus = std::sqrt(1.0f - (cosine * cosine));
            float angle = (rnd(key, bounce, 9 + 2 * tries) * 2.0f * PI_F);
            float angleCos = std::cos(angle);
            float angleSin = std::sqrt(1.0f - (angleCos * angleCos));
            sd = (r * cosine) + (((a * angleCos) + (b * angleSin)) * sinus);
            if (dot(sd, normal) >= 0.0f) break;
        }
        dir = sd;
        type = 1;
        return true;
    }
    V3 sd = point_on_sphere(rnd(key, bounce, 1), rnd(key, bounce, 2), 1.0f);
    if (dot(sd, normal) < 0.0f) sd = sd * -1.0f;
    dir = sd;
    type = 2;
    return true;
}

// DumbBasedShader::getReflectedColor (DumbBasedShader.impl.cuh:63-122); photon colour factored out
// (the result is linear in it).  `direct` selects PHOTON_TYPE_DIRECT_ILLUMINATION.
Col dumb_based_reflect(const Scene &S, int tri, const dr_material &m, const Tri &v, const Tri &nt, V3 hit, V3 photon_dir,
                       V3 observer, bool direct, int sample_type, bool &passthrough) {
    passthrough = false;
    V3 masses = get_masses(v, hit);
    const bool textured = any_texture(m);
    const UV uv = textured ? hit_uv(S, tri, masses) : UV{0.0f, 0.0f};
    if (textured && cut_out(S, m, uv)) {
        const float pass = (dot(normalized(observer), normalized(photon_dir)) >= 0.9999f) ? 1.0f : 0.0f;
        return Col{pass, pass, pass};
    }
    if (dot(normalized(tri_normal(v)), photon_dir) > 0.0f)
        if (!direct) { passthrough = true; return Col{1, 1, 1}; }
    if (dot(mass_center(nt, masses), observer) < 0.0f) return Col{0, 0, 0};
    V3 n = shading_normal(S, m, tri, v, nt, masses, uv);
    V3 wi = -normalized(photon_dir);
    float metal = std::fmax(std::fmin(m.metal, 1.0f), 0.0f);
    float spec = m.specular;
    Col brdf{0, 0, 0};
    bool brdfMatters = (direct || sample_type == 1);
    if (brdfMatters) {
        V3 w0 = normalized(observer);
        V3 wh = normalized(w0 + wi);
        Col fres = col(m.fresnel);
        if (m.texture[DR_TEX_FRESNEL] > 0) {
            const F4 t = channel_texel(S, m, DR_TEX_FRESNEL, uv);
            fres = Col{fres.r * t.x, fres.g * t.y, fres.b * t.z};
        }
        float val = (1.0f - dot(wh, wi));
        float sq = val * val;
        Col fwi = fres + (Col{1 - fres.r, 1 - fres.g, 1 - fres.b} * (sq * sq * val));
        float multiplier;
        if (direct) {
            float dwh = ((spec + 2) / (2.0f * PI_F)) * std::pow(dot(n, wh), spec);
            float gwiw0 = std::fmin(1.0f, std::fmin(2.0f * dot(n, wh) * dot(n, w0) / dot(w0, wh), 2.0f * dot(n, wh) * dot(n, wi) / dot(w0, wh)));
            multiplier = (dwh * gwiw0) / (4.0f * dot(n, w0) * dot(n, wi));
        } else multiplier = 1.0f;
        Col bb = fwi * multiplier;
        brdf = Col{std::fmax(0.0f, std::fmin(bb.r, 1.0f)), std::fmax(0.0f, std::fmin(bb.g, 1.0f)), std::fmax(0.0f, std::fmin(bb.b, 1.0f))};
    }
    bool diffuseMatters = (direct || sample_type == 2);
    Col diff = col(m.color) * (1.0f - metal);
    if (m.texture[DR_TEX_COLOR] > 0) {
        const F4 t = channel_texel(S, m, DR_TEX_COLOR, uv);
        diff = Col{diff.r * t.x, diff.g * t.y, diff.b * t.z};
    }
    Col diffuse = diffuseMatters ? diff * dot(n, wi) : Col{0, 0, 0};
    if (brdfMatters && diffuseMatters)
        return Col{std::fmax(0.0f, std::fmin((brdf.r * metal) + diffuse.r, 1.0f)),
                   std::fmax(0.0f, std::fmin((brdf.g * metal) + diffuse.g, 1.0f)),
                   std::fmax(0.0f, std::fmin((brdf.b * metal) + diffuse.b, 1.0f))};
    if (brdfMatters) return brdf;
    return diffuse * (1.0f / (1.0f - metal));
}

// SimpleStochasticShader (SimpleStochasticShader.impl.cuh:4-37)
void ss_params(const dr_material &m, float &diff, float &gloss) {
    float total = m.diffuse + m.smoothness;
    float mul = ((total > 1.0f) ? (1.0f / total) : 1.0f);
    diff = m.diffuse * mul;
    gloss = m.smoothness * mul;
}
V3 ss_request(const dr_material &m, const Tri &v, const Tri &nt, V3 hit, V3 raydir, uint32_t key, uint32_t bounce) {
    float diff, gloss;
    ss_params(m, diff, gloss);
    V3 direction = point_on_sphere(rnd(key, bounce, 1), rnd(key, bounce, 2), 1.0f);
    if (dot(direction, tri_normal(v)) < 0) direction = -direction;
    V3 hn = mass_center(nt, get_masses(v, hit));
    V3 refl = reflection(raydir, hn);
    return normalized((direction * diff) + (refl * gloss));
}
Col ss_reflect(const dr_material &m, const Tri &v, const Tri &nt, V3 hit, V3 photon_dir, V3 observer) {
    float diff, gloss;
    ss_params(m, diff, gloss);
    V3 hn = mass_center(nt, get_masses(v, hit));
    V3 refl = reflection(photon_dir, hn);
    float rc = dot(refl, hn) / std::sqrt(sqrmag(refl) * sqrmag(hn));
    if (rc < 0.0f) rc = 0.0f;
    float oc = dot(observer, refl) / std::sqrt(sqrmag(observer) * sqrmag(refl));
    if (oc < 0.0f) oc = 0.0f;
    return col(m.color) * ((diff * rc) + (gloss * std::pow(oc, m.shininess)));
}

// Shaders::FresnelShader::getReflectedColor (FresnelShader.impl.cuh:14-19, DumbStructs.cuh:136-140):
// Schlick term of the interpolated (not normalised) normal and the reversed photon direction.
Col fresnel_reflect(const Scene &S, int tri, const dr_material &m, const Tri &v, const Tri &nt, V3 hit, V3 photon_dir) {
    V3 masses = get_masses(v, hit);
    V3 light = -normalized(photon_dir);
    V3 normal = mass_center(nt, masses);
    Col c = col(m.color);
    if (m.texture[DR_TEX_COLOR] > 0) {
        const F4 t = channel_texel(S, m, DR_TEX_COLOR, hit_uv(S, tri, masses));
        c = Col{c.r * t.x, c.g * t.y, c.b * t.z};
    }
    float val = (1.0f - dot(normal, light));
    float sq = (val * val);
    float f = sq * sq * val;
    return Col{c.r + ((1.0f - c.r) * f), c.g + ((1.0f - c.g) * f), c.b + ((1.0f - c.b) * f)};
}

// DefaultShaderGeneric (DefaultShader.impl.cuh:3-52): the sample is the reflection of the ray about
// the interpolated normal; the reflected colour uses the observer (hit + direction) - hit.
V3 default_request(const Tri &v, const Tri &nt, V3 hit, V3 raydir) { return reflection(raydir, mass_center(nt, get_masses(v, hit))); }
Col default_reflect(const dr_material &m, const Tri &v, const Tri &nt, V3 hit, V3 photon_dir, V3 observer) {
    float diff, gloss;
    ss_params(m, diff, gloss);
    V3 normal = mass_center(nt, get_masses(v, hit));
    V3 cam = (hit + observer) - hit;
    V3 refl = reflection(photon_dir, normal);
    float cosL = std::fmax(dot(refl, normal) / std::sqrt(sqrmag(refl) * sqrmag(normal)), 0.0f);
    float oc = std::fmax(dot(refl, cam) / std::sqrt(sqrmag(refl) * sqrmag(cam)), 0.0f);
    return col(m.color) * ((diff * cosL) + (gloss * std::pow(oc, m.shininess)));
}

// Material::getReflectedColor dispatch; photon colour factored out.
Col reflect(const Scene &S, int tri, V3 hit, V3 photon_dir, V3 observer, bool direct, int sample_type, bool &pass) {
    const dr_material &m = S.mats[S.mat[tri]];
    pass = false;
    if (m.type == DR_MAT_DUMB_BASED)
        return dumb_based_reflect(S, tri, m, S.tree.tri[tri], S.nrm[tri], hit, photon_dir, observer, direct, sample_type, pass);
    if (m.type == DR_MAT_FRESNEL) return fresnel_reflect(S, tri, m, S.tree.tri[tri], S.nrm[tri], hit, photon_dir);
    if (m.type == DR_MAT_DEFAULT) return default_reflect(m, S.tree.tri[tri], S.nrm[tri], hit, photon_dir, observer);
    return ss_reflect(m, S.tree.tri[tri], S.nrm[tri], hit, photon_dir, observer);
}

// Spotlight::getVertexPhotons, photon k (Spotlight.impl.cuh:35-77); false where the reference skips
// the photon.  Random dimensions 4096 + 64 li + 3 k.
bool spot_photon(const dr_light &l, const Spot &sp, V3 point, uint32_t key, uint32_t bounce, int li, int k, V3 &o, V3 &d,
                 Col &c) {
    const uint32_t d0 = 4096u + 64u * (uint32_t)li + 3u * (uint32_t)k;
    const V3 dir = sp.direction;
    V3 non_dir = (dir.z > 0.9f) ? v3(1.0f, 0.0f, 0.0f) : v3(0.0f, 0.0f, 1.0f);
    V3 ver = normalized(cross(dir, non_dir));
    V3 hor = cross(dir, ver);
    V3 pos;
    if (sp.sphere) {
        pos = point_on_sphere(rnd(key, bounce, d0), rnd(key, bounce, d0 + 1), sp.emitter);
        pos = pos * rnd(key, bounce, d0 + 2);
        pos = pos + col3(l.position);
    } else {
        float angle = (rnd(key, bounce, d0) * ((2.0f * PI_F) - 0.0f)) + 0.0f;
        V3 ring = (ver * std::cos(angle)) + (hor * std::sin(angle));
        pos = col3(l.position) + ((ring * sp.emitter) * std::sqrt(rnd(key, bounce, d0 + 1)));
    }
    V3 delta = point - pos;
    float sqr_distance = sqrmag(delta);
    if (sqr_distance < EPS) return false;
    float distance = std::sqrt(sqr_distance);
    float base = (sp.emitter * sp.emitter);
    float spread = std::fmax(1.0f - sp.outer_cos, EPS);
    float surface = ((sp.sphere ? 0.0f : base) + (sqr_distance * spread));
    float s = (base / (((float)sp.samples) * surface));
    c = sp.color * s;
    float inv = 1.0f / distance;
    V3 dd = delta * inv;
    float cosine = dot(dd, dir);
    if (cosine < sp.inner_cos) {
        if (cosine < sp.outer_cos) return false;
        float a = ((sp.inner_cos - cosine) / (sp.inner_cos - sp.outer_cos));
        float b = (1.0f - a);
        c = c * std::pow((a * b * b) + (b * (1.0f - (a * a))), sp.falloff);
    }
    o = pos;
    d = dd;
    return true;
}

// Light::getVertexPhotons: photon ray (origin, direction) and colour for a shading point.
void light_photon(const dr_light &l, V3 point, uint32_t key, uint32_t bounce, int li, V3 &o, V3 &d, Col &c) {
    uint32_t d0 = 72 + 3 * (uint32_t)li;
    if (l.type == DR_LIGHT_SPHERICAL) {
        V3 ep = point_on_sphere(rnd(key, bounce, d0), rnd(key, bounce, d0 + 1), l.radius);
        ep = ep * rnd(key, bounce, d0 + 2);
        ep = ep + col3(l.position);
        V3 delta = point - ep;
        o = ep;
        d = normalized(delta);
        float inv = 1.0f / sqrmag(delta);
        c = Col{l.color[0] * inv, l.color[1] * inv, l.color[2] * inv};
    } else if (l.type == DR_LIGHT_SOFT_DIRECTIONAL) {
        V3 dir = normalized(col3(l.direction));
        float soft = l.distance * l.softness;
        float rad = soft * rnd(key, bounce, d0);
        V3 off = point_on_sphere(rnd(key, bounce, d0 + 1), rnd(key, bounce, d0 + 2), rad);
        V3 origin = (point - (dir * l.distance)) + off;
        o = origin;
        d = point - origin;
        c = col(l.color);
    } else {
        V3 dir = normalized(col3(l.direction));
        o = point - (dir * l.distance);
        d = dir;
        c = col(l.color);
    }
}

}  // namespace

// --------------------------------------------------------------------------------------------
// Reference-semantics renderer (DumbRenderer.cu:174-443), restated as one forward path per
// sub-pixel sample: with one camera sample and one indirect sample per hit, the reference's layer
// stack is a single chain, and getReflectedColor is linear in the photon colour, so the layer
// gather equals a forward product of per-bounce weights.
namespace {

struct Cam {
    dr_camera c;
    float x;  // 0.5 / tan(angle / 2) for the pinhole lenses
};

// Pixel position in screen space (DumbRenderer.cu:190-217) for boxing mode
float pixel_size(int W, int H, int boxing) {
    float w = (float)W, h = (float)H;
    if (boxing == DR_BOXING_HEIGHT) return 1.0f / h;
    if (boxing == DR_BOXING_WIDTH) return 1.0f / w;
    if (boxing == DR_BOXING_MIN) return 1.0f / ((h <= w) ? h : w);
    if (boxing == DR_BOXING_MAX) return 1.0f / ((h >= w) ? h : w);
    return 1.0f;
}

V3 cam_dir(const dr_camera &c, V3 d) {
    return v3(d.x * c.right[0] + d.y * c.up[0] + d.z * c.forward[0], d.x * c.right[1] + d.y * c.up[1] + d.z * c.forward[1],
              d.x * c.right[2] + d.y * c.up[2] + d.z * c.forward[2]);
}

// Lense::getPixelSamples for the three reference lenses, camera->world applied.
void ref_lens(const Cam &cam, float sx, float sy, float pdx, float pdy, uint32_t key, V3 &o, V3 &d, Col &filter) {
    const dr_camera &c = cam.c;
    filter = Col{1, 1, 1};
    if (c.lens == DR_LENS_DEFAULT_PERSPECTIVE) {
        o = v3(0, 0, 0);
        d = normalized(v3(sx, sy, cam.x));
    } else if (c.lens == DR_LENS_SIMPLE_STOCHASTIC) {
        float ox = pdx / 2.0f, oy = pdy / 2.0f;
        float jx = (rnd(key, LENS_BOUNCE, 0) * (ox - (-ox))) + (-ox);
        float jy = (rnd(key, LENS_BOUNCE, 1) * (oy - (-oy))) + (-oy);
        o = v3(0, 0, 0);
        d = v3(sx + jx, sy + jy, cam.x);
    } else {
        float ox = pdx / 2.0f, oy = pdy / 2.0f;
        float jx = (rnd(key, LENS_BOUNCE, 0) * (ox - (-ox))) + (-ox);
        float jy = (rnd(key, LENS_BOUNCE, 1) * (oy - (-oy))) + (-oy);
        float ha = ((sx + jx) * c.angle[0] / RADIAN_F);
        float va = ((sy + jy) * c.angle[1] / RADIAN_F);
        V3 td = v3(std::sin(ha) * std::cos(va), std::sin(va), std::cos(ha) * std::cos(va));
        V3 target = td * c.focal_distance;
        float ra = (rnd(key, LENS_BOUNCE, 2) * (2.0f * PI_F - 0.0f)) + 0.0f;
        V3 origin = (v3(std::cos(ra), std::sin(ra), 0.0f) * std::asin(rnd(key, LENS_BOUNCE, 3))) * c.softness;
        o = origin;
        d = normalized(target - origin);
        filter = col(c.filter);
    }
    if (c.origin_rows)
        o = v3(o.x * c.row_x[0] + o.y * c.row_x[1] + o.z * c.row_x[2] + c.position[0],
               o.x * c.row_y[0] + o.y * c.row_y[1] + o.z * c.row_y[2] + c.position[1],
               o.x * c.row_z[0] + o.y * c.row_z[1] + o.z * c.row_z[2] + c.position[2]);
    else
        o = cam_dir(c, o) + col3(c.position);
    d = cam_dir(c, d);
}

// One sub-pixel sample of the reference estimator.
Col ref_path(const Scene &S, const Cam &cam, const dr_render_params &p, float sx, float sy, float pdx, float pdy, uint32_t key) {
    V3 o, d;
    Col filter;
    ref_lens(cam, sx, sy, pdx, pdy, key, o, d, filter);
    Col total{0, 0, 0};
    Col thr{1, 1, 1};
    int prev = -1;  // restriction object for the layer ray (parent geometry)
    bool clip = p.cull_backfaces != 0;
    for (int layer = 0; layer <= p.max_bounces; layer++) {
        float t;
        V3 hp;
        int hit = S.tree.cast(o, d, clip, prev, t, hp, nullptr, nullptr);
        if (hit < 0) break;
        // indirect sample request (only while layer < maxLayer), DumbRenderer.cu:373-385
        bool have_child = false;
        V3 cd = v3(0, 0, 0);
        int ctype = 0;
        const dr_material &m = S.mats[S.mat[hit]];
        if (layer < p.max_bounces) {
            if (m.type == DR_MAT_DUMB_BASED)
                have_child = dumb_based_request(S, hit, m, S.tree.tri[hit], S.nrm[hit], hp, d, key, (uint32_t)layer, cd, ctype);
            else if (m.type == DR_MAT_FRESNEL)
                have_child = false;
            else if (m.type == DR_MAT_DEFAULT) {
                cd = default_request(S.tree.tri[hit], S.nrm[hit], hp, d);
                ctype = 0;
                have_child = true;
            } else {
                cd = ss_request(m, S.tree.tri[hit], S.nrm[hit], hp, d, key, (uint32_t)layer);
                ctype = 0;
                have_child = true;
            }
        }
        // direct light: photons cast from the light toward the point, DumbRenderer.cu:300-316, 361-428
        Col direct{0, 0, 0};
        for (int li = 0; li < (int)S.lights.size(); li++) {
          const dr_light &L = S.lights[li];
          const bool spot = L.type == DR_LIGHT_SPOTLIGHT;
          const int count = spot ? S.spots[li].samples : 1;
          for (int k = 0; k < count; k++) {
            V3 lo, ld;
            Col lc;
            if (spot) {
                if (!spot_photon(L, S.spots[li], hp, key, (uint32_t)layer, li, k, lo, ld, lc)) continue;
                if (!S.spots[li].shadows) {
                    bool pass;
                    direct = direct + reflect(S, hit, hp, ld, -d, true, 0, pass) * lc;
                    continue;
                }
            } else {
                light_photon(L, hp, key, (uint32_t)layer, li, lo, ld, lc);
            }
            int restrict_obj = -1;
            for (int guard = 0; guard < 64; guard++) {
                float lt;
                V3 lp;
                int lh = S.tree.cast(lo, ld, clip, restrict_obj, lt, lp, nullptr, nullptr);
                if (lh < 0) break;
                if (lh == hit || sqrmag(lp - hp) <= (8.0f * EPS)) {
                    bool pass;
                    Col r = reflect(S, hit, hp, ld, -d, true, 0, pass);
                    direct = direct + r * lc;
                    break;
                }
                bool pass;
                Col tr = reflect(S, lh, lp, ld, ld, true, 0, pass);
                tr = tr * lc;
                if ((tr.r + tr.g + tr.b) > EPS) {
                    lc = tr;
                    lo = lp + normalized(ld) * (64.0f * EPS);
                    restrict_obj = lh;
                } else break;
            }
          }
        }
        total = total + thr * direct;
        if (!have_child) break;
        // weight the child's colour will receive when its layer is gathered (DumbRenderer.cu:330-345)
        bool pass;
        Col w = reflect(S, hit, hp, -cd, -d, false, ctype, pass);
        thr = thr * w;
        prev = hit;
        o = hp;
        d = cd;
    }
    return total * filter;
}

// --------------------------------------------------------------------------------------------
// Physical-mode FP64 oracle: unbiased path tracer over emissive triangles (no reference
// counterpart).  Same random-number layout as the device kernels, in double precision.
struct D3 {
    double x, y, z;
};
inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
inline D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, double f) { return D3{a.x * f, a.y * f, a.z * f}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 dcross(D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 dnorm(D3 a) { double l = std::sqrt(ddot(a, a)); return a * (1.0 / l); }
inline D3 tod(V3 a) { return D3{a.x, a.y, a.z}; }
inline V3 tof(D3 a) { return V3{(float)a.x, (float)a.y, (float)a.z}; }
const double PI_D = 3.14159265358979323846;

// Physical-mode hit: closest front/back hit; exact same traversal as the reference cast with
// culling off (the float predicate decides visibility, the shading math is double).
void onb(D3 n, D3 &t, D3 &b) {
    double s = n.z >= 0 ? 1.0 : -1.0;
    double a = -1.0 / (s + n.z);
    double bb = n.x * n.y * a;
    t = d3(1.0 + s * n.x * n.x * a, s * bb, -s * n.x);
    b = d3(bb, s + n.y * n.y * a, -n.y);
}

double ggx_d(double ndh, double a) {
    double a2 = a * a;
    double c2 = ndh * ndh;
    double den = c2 * (a2 - 1.0) + 1.0;
    return a2 / (PI_D * den * den);
}
double ggx_g1(double ndv, double a) {
    double a2 = a * a;
    return 2.0 * ndv / (ndv + std::sqrt(a2 + (1.0 - a2) * ndv * ndv));
}

struct Emit {
    double pdf_area;  // pdf of picking this point by NEE, per unit area
};

void phys_lens(const Cam &cam, int W, int H, int px, int py, uint32_t key, D3 &o, D3 &d, bool &valid) {
    const dr_camera &c = cam.c;
    double jx = rndd(key, LENS_BOUNCE, 0), jy = rndd(key, LENS_BOUNCE, 1);
    // screen coordinates in units of the image height, +y up
    double sx = ((double)px + jx - 0.5 * W) / (double)H;
    double sy = (0.5 * H - ((double)py + jy)) / (double)H;
    valid = true;
    D3 dl;
    if (c.lens == DR_LENS_FISHEYE) {
        double r = std::sqrt(sx * sx + sy * sy);
        double theta = r * (c.angle[0] * PI_D / 180.0);  // r = 0.5 at the top edge -> half the fov
        if (theta > PI_D) { valid = false; o = d3(0, 0, 0); d = d3(0, 0, 1); return; }
        double phi = std::atan2(sy, sx);
        double st = std::sin(theta);
        dl = d3(st * std::cos(phi), st * std::sin(phi), std::cos(theta));
    } else if (c.lens == DR_LENS_SPHERICAL) {
        double h = sx * (c.angle[0] * PI_D / 180.0);
        double v = sy * (c.angle[1] * PI_D / 180.0);
        dl = d3(std::sin(h) * std::cos(v), std::sin(v), std::cos(h) * std::cos(v));
    } else {
        double x = 0.5 / std::tan(c.angle[0] * PI_D / 360.0);
        dl = dnorm(d3(sx, sy, x));
    }
    D3 R = d3(c.right[0], c.right[1], c.right[2]), U = d3(c.up[0], c.up[1], c.up[2]), F = d3(c.forward[0], c.forward[1], c.forward[2]);
    d = dnorm(R * dl.x + U * dl.y + F * dl.z);
    o = d3(c.position[0], c.position[1], c.position[2]);
}

// Geometric normal of triangle i facing `wo` side is decided at shading time.
D3 geo_normal(const Scene &S, int i) {
    const Tri &t = S.tree.tri[i];
    return dnorm(dcross(tod(t.b) - tod(t.a), tod(t.c) - tod(t.a)));
}
double tri_area(const Scene &S, int i) {
    const Tri &t = S.tree.tri[i];
    return 0.5 * std::sqrt(ddot(dcross(tod(t.b) - tod(t.a), tod(t.c) - tod(t.a)), dcross(tod(t.b) - tod(t.a), tod(t.c) - tod(t.a))));
}
double emit_power(const Scene &S, int i) {
    return (S.emission[3 * i] + S.emission[3 * i + 1] + S.emission[3 * i + 2]) * tri_area(S, i);
}
// Power that light selection (the NEE table and the light pdf of MIS) uses for triangle i.
double sample_power(const Scene &S, int i) {
    return S.frozen_power.empty() ? emit_power(S, i) : S.frozen_power[i];
}

// Occlusion between p and q (segment strictly between the end points), float cast, no culling.
bool occluded(const Scene &S, D3 p, D3 q, int ignore_a, int ignore_b) {
    V3 o = tof(p);
    V3 d = tof(q - p);
    float t;
    V3 hp;
    // closest hit ignoring the shading triangle; occluded if it lies before the light point
    int h = S.tree.cast(o, d, false, ignore_a, t, hp, nullptr, nullptr);
    if (h < 0) return false;
    if (h == ignore_b) return false;
    return t < 0.999f;
}

// MIS power heuristic
inline double mis2(double a, double b) { return (a * a) / (a * a + b * b); }

void phys_path(const Scene &S, const Cam &cam, int W, int H, int px, int py, int maxb, uint32_t key, double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    D3 o, d;
    bool valid;
    phys_lens(cam, W, H, px, py, key, o, d, valid);
    if (!valid) return;
    double thr[3] = {1, 1, 1};
    int prev = -1;
    double prev_pdf = 0.0;  // solid-angle pdf of the bsdf sample that produced this ray (0 = delta / camera)
    bool prev_delta = true;
    for (int b = 0; b <= maxb; b++) {
        float t;
        V3 hpf;
        int hit = S.tree.cast(tof(o), tof(d), false, prev, t, hpf, nullptr, nullptr);
        if (hit < 0) break;
        D3 hp = o + d * (double)t;
        D3 ng = geo_normal(S, hit);
        D3 wo = d * -1.0;
        if (ddot(ng, wo) < 0) ng = ng * -1.0;
        // emission (one-sided: front = the side the outward normal (c-a)x(b-a) faces)
        const float *em = &S.emission[3 * hit];
        if (em[0] + em[1] + em[2] > 0.0f) {
            const Tri &tt = S.tree.tri[hit];
            D3 outward = dnorm(dcross(tod(tt.c) - tod(tt.a), tod(tt.b) - tod(tt.a)));
            double cosl = ddot(outward, wo);
            if (cosl > 0) {
                double w = 1.0;
                if (!prev_delta && S.emissive_total > 0) {
                    double pl = sample_power(S, hit) / S.emissive_total / tri_area(S, hit);
                    double pls = pl * ((double)t * (double)t * ddot(d, d)) / cosl;
                    w = mis2(prev_pdf, pls);
                }
                for (int k = 0; k < 3; k++) out[k] += thr[k] * em[k] * w;
            }
        }
        if (b == maxb) break;
        int mt = S.mats[S.mat[hit]].type;
        const float *alb = &S.albedo[3 * hit];
        double rough = S.rough[hit];
        double alpha = std::fmax(rough, 1e-3);
        // next-event estimation toward emissive triangles (non-delta materials)
        if (mt != DR_MAT_MIRROR && S.emissive_total > 0) {
            double u = rndd(key, (uint32_t)b, 3) * S.emissive_total;
            int lo = 0, hi = (int)S.emissive_cdf.size() - 1;
            while (lo < hi) { int mid = (lo + hi) / 2; if (S.emissive_cdf[mid] < u) lo = mid + 1; else hi = mid; }
            int li = S.emissive[lo];
            double u1 = rndd(key, (uint32_t)b, 4), u2 = rndd(key, (uint32_t)b, 5);
            double su = std::sqrt(u1);
            double ba = 1.0 - su, bb = u2 * su;
            const Tri &lt = S.tree.tri[li];
            D3 lp = tod(lt.a) * ba + tod(lt.b) * bb + tod(lt.c) * (1.0 - ba - bb);
            D3 ld = lp - hp;
            double dist2 = ddot(ld, ld);
            D3 wi = ld * (1.0 / std::sqrt(dist2));
            D3 lout = dnorm(dcross(tod(lt.c) - tod(lt.a), tod(lt.b) - tod(lt.a)));
            double cosl = -ddot(lout, wi);
            double cosi = ddot(ng, wi);
            if (cosl > 0 && cosi > 0 && !occluded(S, hp, lp, hit, li)) {
                double pl = sample_power(S, li) / S.emissive_total / tri_area(S, li);
                double pls = pl * dist2 / cosl;
                double f[3], pb;
                if (mt == DR_MAT_GLOSSY) {
                    D3 h = dnorm(wi + wo);
                    double ndh = ddot(ng, h), ndo = ddot(ng, wo);
                    double D = ggx_d(ndh, alpha);
                    double G = ggx_g1(ndo, alpha) * ggx_g1(cosi, alpha);
                    double spec = D * G / (4.0 * ndo * cosi);
                    for (int k = 0; k < 3; k++) f[k] = alb[k] * spec;
                    pb = D * ndh / (4.0 * std::fabs(ddot(wo, h)));
                } else {
                    for (int k = 0; k < 3; k++) f[k] = alb[k] / PI_D;
                    pb = cosi / PI_D;
                }
                double w = mis2(pls, pb);
                const float *le = &S.emission[3 * li];
                for (int k = 0; k < 3; k++) out[k] += thr[k] * f[k] * le[k] * cosi / pls * w;
            }
        }
        // bsdf sampling
        double u1 = rndd(key, (uint32_t)b, 1), u2 = rndd(key, (uint32_t)b, 2);
        D3 T, B;
        onb(ng, T, B);
        D3 nd;
        if (mt == DR_MAT_MIRROR) {
            nd = d - ng * (2.0 * ddot(d, ng));
            for (int k = 0; k < 3; k++) thr[k] *= alb[k];
            prev_delta = true;
            prev_pdf = 0.0;
        } else if (mt == DR_MAT_GLOSSY) {
            double phi = 2.0 * PI_D * u1;
            double ct = std::sqrt((1.0 - u2) / (1.0 + (alpha * alpha - 1.0) * u2));
            double st = std::sqrt(std::fmax(0.0, 1.0 - ct * ct));
            D3 h = T * (st * std::cos(phi)) + B * (st * std::sin(phi)) + ng * ct;
            nd = h * (2.0 * ddot(wo, h)) - wo;
            double cosi = ddot(ng, nd);
            if (cosi <= 0) break;
            double ndo = ddot(ng, wo);
            double G = ggx_g1(ndo, alpha) * ggx_g1(cosi, alpha);
            double wgt = G * std::fabs(ddot(wo, h)) / (ndo * ct);
            for (int k = 0; k < 3; k++) thr[k] *= alb[k] * wgt;
            prev_pdf = ggx_d(ct, alpha) * ct / (4.0 * std::fabs(ddot(wo, h)));
            prev_delta = false;
        } else {
            double r = std::sqrt(u1), phi = 2.0 * PI_D * u2;
            double z = std::sqrt(std::fmax(0.0, 1.0 - u1));
            nd = T * (r * std::cos(phi)) + B * (r * std::sin(phi)) + ng * z;
            for (int k = 0; k < 3; k++) thr[k] *= alb[k];
            prev_pdf = z / PI_D;
            prev_delta = false;
        }
        prev = hit;
        o = hp;
        d = dnorm(nd);
    }
}

}  // namespace

// --------------------------------------------------------------------------------------------
extern "C" {

void *dro_scene_create(const float *xyz, const float *nrm, const int *mat, int n, const dr_material *mats, int n_mats,
                       const dr_light *lights, int n_lights, int max_depth, int split_n, int threads) {
    Scene *S = new Scene();
    S->tree.max_depth = max_depth > 0 ? max_depth : 24;
    S->tree.split_n = split_n > 0 ? split_n : 8;
    S->tree.tri.resize(n);
    S->nrm.resize(n);
    S->mat.resize(n);
    for (int i = 0; i < n; i++) {
        const float *p = xyz + 9 * i;
        S->tree.tri[i] = Tri{v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]), v3(p[6], p[7], p[8])};
        if (nrm) {
            const float *q = nrm + 9 * i;
            S->nrm[i] = Tri{v3(q[0], q[1], q[2]), v3(q[3], q[4], q[5]), v3(q[6], q[7], q[8])};
        } else {
            V3 fn = normalized(tri_normal(S->tree.tri[i]));
            S->nrm[i] = Tri{fn, fn, fn};
        }
        S->mat[i] = mat ? mat[i] : 0;
    }
    S->mats.assign(mats, mats + n_mats);
    S->lights.assign(lights, lights + n_lights);
    for (int i = 0; i < n_lights; i++) S->spots.push_back(spot_state(lights[i]));
    S->albedo.resize(3 * (size_t)n);
    S->emission.assign(3 * (size_t)n, 0.0f);
    S->rough.resize(n);
    for (int i = 0; i < n; i++) {
        const dr_material &m = S->mats.empty() ? dr_material{} : S->mats[S->mat[i]];
        for (int k = 0; k < 3; k++) { S->albedo[3 * i + k] = m.color[k]; S->emission[3 * i + k] = m.emission[k]; }
        S->rough[i] = m.roughness;
    }
    S->tree.build(threads > 0 ? threads : (int)std::thread::hardware_concurrency());
    return S;
}

// Textures and per-corner texture coordinates (float[n][3][2] or NULL for zeros), as dr_scene_set_textures.
void dro_scene_set_textures(void *h, const dr_texture *tex, int n, const float *uv) {
    Scene *S = (Scene *)h;
    S->tex.clear();
    for (int i = 0; i < n; i++) {
        Scene::Tex t{tex[i].width, tex[i].height, tex[i].filtering, {}};
        t.rgba.assign(tex[i].rgba, tex[i].rgba + 4 * (size_t)tex[i].width * (size_t)tex[i].height);
        S->tex.push_back(std::move(t));
    }
    S->uv.assign(6 * S->tree.tri.size(), 0.0f);
    if (uv) std::memcpy(S->uv.data(), uv, sizeof(float) * S->uv.size());
}

void dro_scene_set_triangle_params(void *h, const float *albedo, const float *emission, const float *rough) {
    Scene *S = (Scene *)h;
    size_t n = S->tree.tri.size();
    if (albedo) std::memcpy(S->albedo.data(), albedo, 12 * n);
    if (emission) std::memcpy(S->emission.data(), emission, 12 * n);
    if (rough) std::memcpy(S->rough.data(), rough, 4 * n);
}

// freeze != 0: light selection keeps the current per-triangle emission power from now on, whatever
// later parameter updates write (finite differences with common random numbers then differentiate
// a fixed estimator); freeze == 0: it follows the current emission again.
void dro_scene_freeze_sampling(void *h, int freeze) {
    Scene *S = (Scene *)h;
    S->frozen_power.clear();
    if (!freeze) return;
    S->frozen_power.resize(S->tree.tri.size());
    for (int i = 0; i < (int)S->tree.tri.size(); i++) S->frozen_power[i] = emit_power(*S, i);
}

static void build_emissive(Scene *S) {
    S->emissive.clear();
    S->emissive_cdf.clear();
    S->emissive_total = 0.0;
    for (int i = 0; i < (int)S->tree.tri.size(); i++) {
        double p = sample_power(*S, i);
        if (p > 0) { S->emissive.push_back(i); S->emissive_total += p; S->emissive_cdf.push_back(S->emissive_total); }
    }
}

void dro_scene_destroy(void *h) { delete (Scene *)h; }

long long dro_node_count(void *h) { return (long long)((Scene *)h)->tree.nodes.size(); }

// Flattened tree (node i: box, first child or -1, leaf list) for structural comparison.
// Node order: the oracle's own order, not comparable index-by-index with other builders.
void dro_tree_stats(void *h, long long *nodes, long long *leaves, long long *refs, int *depth) {
    Scene *S = (Scene *)h;
    long long nl = 0, nr = 0;
    int dmax = 0;
    std::vector<std::pair<int, int>> st{{0, 0}};
    while (!st.empty()) {
        auto [i, dep] = st.back();
        st.pop_back();
        dmax = std::max(dmax, dep);
        const Node &nd = S->tree.nodes[i];
        if (nd.child < 0) { nl++; nr += (long long)nd.tris.size(); }
        else for (int k = 0; k < 8; k++) st.push_back({nd.child + k, dep + 1});
    }
    *nodes = (long long)S->tree.nodes.size();
    *leaves = nl;
    *refs = nr;
    *depth = dmax;
}

// Canonical tree dump: depth-first in child order; per node 6 floats + leaf count, followed by
// the leaf's triangle ids.  Lets two builders be compared independent of node numbering.
long long dro_tree_canonical(void *h, float *boxes, int *counts, int *tris, long long cap_nodes, long long cap_refs) {
    Scene *S = (Scene *)h;
    long long k = 0, r = 0;
    std::vector<int> st{0};
    while (!st.empty()) {
        int i = st.back();
        st.pop_back();
        const Node &nd = S->tree.nodes[i];
        if (k < cap_nodes) {
            float *b = boxes + 6 * k;
            b[0] = nd.b.s.x; b[1] = nd.b.s.y; b[2] = nd.b.s.z; b[3] = nd.b.e.x; b[4] = nd.b.e.y; b[5] = nd.b.e.z;
            counts[k] = nd.child < 0 ? (int)nd.tris.size() : -1;
        }
        k++;
        if (nd.child < 0) {
            for (int id : nd.tris) { if (r < cap_refs) tris[r] = id; r++; }
        } else
            for (int c = 7; c >= 0; c--) st.push_back(nd.child + c);
    }
    return k;
}

void dro_cast(void *h, const float *o, const float *d, const int *ignore, int n, int clip, int threads, int *idx, float *t,
              int *boxes, int *tests) {
    Scene *S = (Scene *)h;
    if (threads < 1) threads = 1;
    auto work = [&](int tid) {
        for (int i = tid; i < n; i += threads) {
            long long nb = 0, nt = 0;
            float tt = FLT_MAX;
            V3 hp;
            int hi = S->tree.cast(v3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), v3(d[3 * i], d[3 * i + 1], d[3 * i + 2]), clip != 0,
                                  ignore ? ignore[i] : -1, tt, hp, &nb, &nt);
            idx[i] = hi;
            t[i] = hi >= 0 ? tt : FLT_MAX;
            if (boxes) boxes[i] = (int)nb;
            if (tests) tests[i] = (int)nt;
        }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < threads; k++) pool.emplace_back(work, k);
    work(0);
    for (auto &th : pool) th.join();
}

// Renders blocks [start, end) of the image in the reference's block-major layout, setting or
// blending (1/iteration) each pixel, with the same counter-based random numbers as the device
// renderer.  Reference semantics (mode 0, float) or physical mode (mode 1, double).
void dro_render_blocks(void *h, const dr_camera *camera, const dr_render_params *p, float *fb, int start, int end, int threads) {
    Scene *S = (Scene *)h;
    if (p->mode == DR_MODE_PHYSICAL) build_emissive(S);
    Cam cam;
    cam.c = *camera;
    {
        float angle = camera->angle[0];
        if (angle < 1) angle = 1;
        else if (angle > 179) angle = 179;
        float radian = (angle / (2 * RADIAN_F));
        cam.x = (camera->lens_x > 0.0f) ? camera->lens_x : 0.5f / std::tan(radian);
    }
    int W = p->width, H = p->height;
    int bw = (W + DR_BLOCK_W - 1) / DR_BLOCK_W;
    int fx = p->samples_x < 1 ? 1 : p->samples_x, fy = p->samples_y < 1 ? 1 : p->samples_y;
    float ps = pixel_size(W, H, p->boxing);
    float pdx = ps / (float)fx, pdy = ps / (float)fy;
    float blend = (p->iteration <= 1) ? 1.0f : (1.0f / (float)p->iteration);
    int spp = fx * fy;
    uint32_t sample_base = (uint32_t)((p->iteration < 1 ? 0 : p->iteration - 1) * spp);
    if (threads < 1) threads = 1;
    std::atomic<int> next{start};
    auto work = [&]() {
        for (;;) {
            int blk = next.fetch_add(1);
            if (blk >= end) break;
            int by = blk / bw, bx = blk - by * bw;
            for (int pid = 0; pid < DR_BLOCK_W * DR_BLOCK_H; pid++) {
                int oy = pid / DR_BLOCK_W, ox = pid - oy * DR_BLOCK_W;
                int x = bx * DR_BLOCK_W + ox, y = by * DR_BLOCK_H + oy;
                if (x >= W || y >= H) continue;
                uint32_t pixel = (uint32_t)(y * W + x);
                float acc[3] = {0, 0, 0};
                if (p->mode == DR_MODE_PHYSICAL) {
                    double a[3] = {0, 0, 0};
                    for (int s = 0; s < spp; s++) {
                        uint32_t key = path_key(p->seed, pixel, sample_base + (uint32_t)s);
                        double c[3];
                        phys_path(*S, cam, W, H, x, y, p->max_bounces, key, c);
                        for (int k = 0; k < 3; k++) a[k] += c[k];
                    }
                    for (int k = 0; k < 3; k++) acc[k] = (float)(a[k] / spp);
                } else {
                    float px = ((float)x - ((float)W / 2.0f)) * ps;
                    float py = (((float)H / 2.0f) - (float)y) * ps;
                    float sw = 1.0f / (((float)fx) * ((float)fy));
                    int s = 0;
                    for (int i = 0; i < fx; i++)
                        for (int j = 0; j < fy; j++, s++) {
                            float sx = px + (((float)i) + 0.5f) * pdx;
                            float sy = py + (((float)j) + 0.5f) * pdy;
                            uint32_t key = path_key(p->seed, pixel, sample_base + (uint32_t)s);
                            Col c = ref_path(*S, cam, *p, sx, sy, pdx, pdy, key);
                            acc[0] += c.r * sw; acc[1] += c.g * sw; acc[2] += c.b * sw;
                        }
                }
                float *dst = fb + 4 * ((size_t)blk * (DR_BLOCK_W * DR_BLOCK_H) + pid);
                if (blend >= 1.0f) { dst[0] = acc[0]; dst[1] = acc[1]; dst[2] = acc[2]; dst[3] = 1.0f; }
                else {
                    for (int k = 0; k < 3; k++) dst[k] = (acc[k] * blend) + (dst[k] * (1.0f - blend));
                    dst[3] = (1.0f * blend) + (dst[3] * (1.0f - blend));
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < threads; k++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
}

uint32_t dro_rng_u32(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t bounce, uint32_t dim) {
    uint32_t key = path_key(seed, pixel, sample);
    return hash32(hash32(key + 0x9E3779B9U * (bounce * 128U + dim + 1U)));
}

}  // extern "C"
