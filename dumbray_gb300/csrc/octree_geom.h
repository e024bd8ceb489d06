// octree_geom.h - the geometry of the octree build (triangle/box clipping, overlap, clipped centres
// and bounds, octant and shrink boxes), shared by the host builder (g++, -ffp-contract=off) and the
// device builder (nvcc, -fmad=false): both execute the same IEEE single-precision operations in the
// same order, so they build bit-identical trees.
//
// The operations restate the reference's (Octree.impl.cuh:423-434 splitAABB, :489-533 reduceNode;
// AABB.impl.h:152-221 intersectsTri; Shapes.impl.cuh:178-310 clipped intersections, their bounds and
// area-weighted centres; Triangle.impl.h:183-196 sortByMases).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define DRB_HD __host__ __device__ __forceinline__
#else
#define DRB_HD inline
#endif

namespace drb {
namespace geom {

struct P3 {
    float x, y, z;
};
DRB_HD P3 mk(float x, float y, float z) { return P3{x, y, z}; }
DRB_HD P3 add(P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; }
DRB_HD P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
DRB_HD P3 scale(P3 a, float f) { return P3{a.x * f, a.y * f, a.z * f}; }
DRB_HD P3 divs(P3 a, float f) {
    float r = 1.0f / f;
    return P3{a.x * r, a.y * r, a.z * r};
}
DRB_HD P3 crs(P3 a, P3 v) { return P3{a.y * v.z - v.y * a.z, v.x * a.z - a.x * v.z, a.x * v.y - v.x * a.y}; }
DRB_HD float len(P3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
DRB_HD float comp(P3 v, int ax) { return ax == 0 ? v.x : (ax == 1 ? v.y : v.z); }
DRB_HD float fmin_(float a, float b) { return fminf(a, b); }
DRB_HD float fmax_(float a, float b) { return fmaxf(a, b); }
template <class T>
DRB_HD void swap_(T &a, T &b) {
    T t = a;
    a = b;
    b = t;
}

struct Bx {
    P3 lo, hi;
};
DRB_HD Bx fixed_box(P3 s, P3 e) {
    if (s.x > e.x) swap_(s.x, e.x);
    if (s.y > e.y) swap_(s.y, e.y);
    if (s.z > e.z) swap_(s.z, e.z);
    return Bx{s, e};
}

struct T3 {
    P3 a, b, c;
};

// Vertex order by one axis.
DRB_HD void order_by(T3 &t, int ax) {
    float am = comp(t.a, ax), bm = comp(t.b, ax), cm = comp(t.c, ax);
    if (am > bm) {
        if (cm > am) swap_(t.a, t.b);
        else if (bm > cm) swap_(t.a, t.c);
        else { P3 k = t.a; t.a = t.b; t.b = t.c; t.c = k; }
    } else {
        if (am > cm) { P3 k = t.a; t.a = t.c; t.c = t.b; t.b = k; }
        else if (bm > cm) swap_(t.b, t.c);
    }
}
DRB_HD P3 lerp_at(P3 from, P3 to, float fv, float tv, float plane) { return add(from, scale(sub(to, from), (plane - fv) / (tv - fv))); }

// Piecewise slab clipping of one triangle against [s, e] on axis `ax`, emitting pieces through
// `emit`; returns early (true) as soon as `emit` returns true.  Serves both the exact overlap test
// (stops on the first surviving piece) and the clipping behind intersection centres and bounds.
template <class Emit>
DRB_HD bool slab_clip(T3 t, int ax, float s, float e, Emit &emit) {
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
struct AnyPiece {
    DRB_HD bool operator()(const T3 &) const { return true; }
};
struct YLevel {
    const Bx *b;
    DRB_HD bool operator()(const T3 &p) const {
        AnyPiece any;
        return slab_clip(p, 1, b->lo.y, b->hi.y, any);
    }
};
struct XLevel {
    const Bx *b;
    DRB_HD bool operator()(const T3 &p) const {
        YLevel y{b};
        return slab_clip(p, 0, b->lo.x, b->hi.x, y);
    }
};
DRB_HD bool overlaps(const Bx &b, const T3 &t) {
    XLevel x{&b};
    return slab_clip(t, 2, b.lo.z, b.hi.z, x);
}

// All pieces of t inside b (x, then y, then z), in the reference's order (at most 32 kept per stage).
struct Pieces {
    T3 p[32];
    int n;
};
struct Collect {
    Pieces *dst;
    DRB_HD bool operator()(const T3 &p) const {
        if (dst->n < 32) dst->p[dst->n++] = p;
        return false;
    }
};
DRB_HD void clip_all(const Bx &b, const T3 &t, Pieces &out, Pieces &x, Pieces &y) {
    x.n = 0;
    y.n = 0;
    out.n = 0;
    Collect cx{&x}, cy{&y}, cz{&out};
    slab_clip(t, 0, b.lo.x, b.hi.x, cx);
    for (int i = 0; i < x.n; i++) slab_clip(x.p[i], 1, b.lo.y, b.hi.y, cy);
    for (int i = 0; i < y.n; i++) slab_clip(y.p[i], 2, b.lo.z, b.hi.z, cz);
}

// Area-weighted centre of the clipped pieces (box centre when nothing is left).
DRB_HD P3 clipped_centre(const Bx &b, const T3 &t, Pieces &l, Pieces &x, Pieces &y) {
    clip_all(b, t, l, x, y);
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

// Bounds of the clipped pieces (the box itself when nothing is left).
DRB_HD Bx clipped_bounds(const Bx &b, const T3 &t, Pieces &l, Pieces &x, Pieces &y) {
    clip_all(b, t, l, x, y);
    if (l.n == 0) return b;
    P3 lo = b.hi, hi = b.lo;
    for (int i = 0; i < l.n; i++) {
        const T3 &p = l.p[i];
        const P3 v[3] = {p.a, p.b, p.c};
        for (int k = 0; k < 3; k++)
            hi = mk(hi.x > v[k].x ? hi.x : v[k].x, hi.y > v[k].y ? hi.y : v[k].y, hi.z > v[k].z ? hi.z : v[k].z);
        for (int k = 0; k < 3; k++)
            lo = mk(lo.x < v[k].x ? lo.x : v[k].x, lo.y < v[k].y ? lo.y : v[k].y, lo.z < v[k].z ? lo.z : v[k].z);
    }
    return fixed_box(lo, hi);
}

// The 8 overlapping octants around `c` padded by E; child bit 2 = upper x, 1 = upper y, 0 = upper z.
DRB_HD void octants(const Bx &b, P3 c, Bx *r, float E) {
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

// Shrink a node box to lo..hi padded by E, clamped to the old box.
DRB_HD Bx shrink(const Bx &old, P3 lo, P3 hi, float E) {
    lo = sub(lo, mk(E, E, E));
    hi = add(hi, mk(E, E, E));
    lo = mk(fmax_(lo.x, old.lo.x), fmax_(lo.y, old.lo.y), fmax_(lo.z, old.lo.z));
    hi = mk(fmin_(hi.x, old.hi.x), fmin_(hi.y, old.hi.y), fmin_(hi.z, old.hi.z));
    return fixed_box(lo, hi);
}

// Triangle bounds: padded by E except for the first triangle (the root box rule of push).
DRB_HD Bx tri_box(const T3 &t) {
    P3 lo = mk(t.a.x < t.b.x ? t.a.x : t.b.x, t.a.y < t.b.y ? t.a.y : t.b.y, t.a.z < t.b.z ? t.a.z : t.b.z);
    lo = mk(lo.x < t.c.x ? lo.x : t.c.x, lo.y < t.c.y ? lo.y : t.c.y, lo.z < t.c.z ? lo.z : t.c.z);
    P3 hi = mk(t.a.x > t.b.x ? t.a.x : t.b.x, t.a.y > t.b.y ? t.a.y : t.b.y, t.a.z > t.b.z ? t.a.z : t.b.z);
    hi = mk(hi.x > t.c.x ? hi.x : t.c.x, hi.y > t.c.y ? hi.y : t.c.y, hi.z > t.c.z ? hi.z : t.c.z);
    return fixed_box(lo, hi);
}

}  // namespace geom
}  // namespace drb
