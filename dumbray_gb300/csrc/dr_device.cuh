// dr_device.cuh - device-side scene layout and the exact octree cast for sm_103a.
//
// Layout in HBM (all read-only after upload):
//   nodes      float4[2 * node_count]  node i = {lo.xyz, w = first child (inner) or ~first ref (leaf)},
//                                               {hi.xyz, w = leaf ref count}
//              children of an inner node are 8 consecutive nodes, 8-aligned (one 256-byte group).
//   leaf_tris  float4[3 * refs]        leaf reference r = {a.xyz, w = triangle id}, {b.xyz}, {c.xyz}:
//              the leaf's triangles duplicated in leaf order, so a leaf is one contiguous stream.
//   tris       float4[3 * n]           triangles by id (shading, light sampling)
// The cast reproduces DumbRay's Octree::cast (Octree.impl.cuh:174-212) bit for bit: every
// floating-point operation of the slab test, the triangle plane test and the edge-angle
// containment predicate is issued as an explicitly rounded intrinsic (__fadd_rn, __fmul_rn,
// __fdiv_rn, __fsqrt_rn), so no FMA contraction or approximate division can change a result.
#pragma once
#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace drd {

constexpr float kEps = 0.000005f;               // VECTOR_EPSILON (Vector3.h:10)
constexpr int kMaxDepth = 24;                    // OCTREE_MAX_DEPTH (Octree.cuh:13)
constexpr int kStack = kMaxDepth + 2;

struct Material {
    int type;
    float color[3];
    float fresnel[3];
    float specular, metal, diffuse, smoothness, shininess, roughness;
    float emission[3];
    int texture[4];              // 0-based texture per channel (colour, fresnel, normal, alpha), -1 = none
    float tiling[4][2], offset[4][2];
    float normal_color[3];
    float alpha_threshold;
};

struct Light {
    int type;
    float color[3];      // spotlight: colour x luminosity
    float position[3];
    float direction[3];  // spotlight: normalised
    float radius, distance, softness;
    // spotlight (Lights::Spotlight constructor state): emitter size, cosines of the hotspot and
    // falloff half-angles, falloff power, photons per shading point, occlusion test, sphere emitter
    float emitter, inner_cos, outer_cos, falloff;
    int samples, shadows, sphere;
};

struct Scene {
    const float4 *nodes;
    // Child boxes per node group as planes of 8 floats (lo.x, lo.y, lo.z, hi.x, hi.y, hi.z; 12 float4
    // = 192 B per group), read by the group tests: 12 vector loads instead of 16.  gbox: refitted to
    // the non-empty leaves below each child (every traversal but the next); gbox_ref: the reference's
    // boxes (counting traversals of reference-padding scenes).  Empty leaves sit at a far point in
    // both (dr_octree_group_planes in the C ABI gives both for a host-built tree).
    const float4 *gbox;
    const float4 *gbox_ref;
    const float4 *leaf_tris;
    const float4 *tris;
    const float4 *nrms;
    const int *mat_id;
    const Material *mats;
    const Light *lights;
    const float4 *shade;        // physical: [n] {roughness, type bits, -, -}
    const float *albedo;        // physical: [n][3] (writable in place by an optimiser)
    const float *emission;      // physical: [n][3] (writable in place; sampling tables are not rebuilt)
    const float *light_pdf;     // physical: [n] area pdf of picking a point of this triangle by NEE
    const int *emissive;        // emissive triangle ids
    const float *emissive_cdf;  // inclusive prefix sums of power (at table build time)
    const float4 *texels;       // all textures' RGBA texels, row-major per texture
    const int4 *tex_info;       // per texture: {first texel, width, height, filtering}
    const float2 *uv;           // [n][3] corner texture coordinates (null: none set)
    float root_lo[3], root_hi[3];
    int root_child;             // node group of the root's 8 children (0 for a standalone scene, the
                                // scene's offset in a batch arena), -1 = the root is a leaf
    int root_leaf_first, root_leaf_count;
    int n_tris, n_mats, n_lights, n_emissive;
    int shadow_photons;  // shadow records one reference-mode hit can emit (1 per light, a spotlight's samples)
    // Boxes lying entirely behind the ray origin: the reference's slab test keeps them
    // (clipBackface = false), which only costs work, since a hit at t > 0 accepted inside a leaf box
    // means that box reaches t > 0.  Every non-counting traversal skips them; the counting ones
    // (which reproduce the reference's box-test counts) skip them only when front_only = 1, i.e. for
    // scenes built with a padding scaled to the scene, whose counts are not the reference's anyway.
    int front_only;
    float emissive_total;
};

// ---- exactly rounded float3 arithmetic (reference operation order) -------------------------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mkf3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 xsub(f3 a, f3 b) { return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 xadd(f3 a, f3 b) { return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 xmul(f3 a, float f) { return f3{__fmul_rn(a.x, f), __fmul_rn(a.y, f), __fmul_rn(a.z, f)}; }
// Vector3 dot: (x*v.x + y*v.y) + z*v.z
__device__ __forceinline__ float xdot(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// Vector3 cross a & v: (y*v.z - v.y*z, v.x*z - x*v.z, x*v.y - v.x*y)
__device__ __forceinline__ f3 xcross(f3 a, f3 v) {
    return f3{__fsub_rn(__fmul_rn(a.y, v.z), __fmul_rn(v.y, a.z)), __fsub_rn(__fmul_rn(v.x, a.z), __fmul_rn(a.x, v.z)),
              __fsub_rn(__fmul_rn(a.x, v.y), __fmul_rn(v.x, a.y))};
}
__device__ __forceinline__ float xmag(f3 a) { return __fsqrt_rn(xdot(a, a)); }
__device__ __forceinline__ bool xeq(f3 a, f3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
__device__ __forceinline__ f3 f3of(float4 v) { return f3{v.x, v.y, v.z}; }

// AABB::castPreInversed + Shapes::castPreInversed<AABB>(.., clipBackface = false)
// (AABB.impl.h:116-130, Shapes.impl.cuh:143-147)
__device__ __forceinline__ bool slab_hit(float lx, float ly, float lz, float hx, float hy, float hz, f3 o, f3 inv,
                                         bool front = false) {
    float ds = __fmul_rn(__fsub_rn(lx, o.x), inv.x);
    float de = __fmul_rn(__fsub_rn(hx, o.x), inv.x);
    float mn = fminf(ds, de), mx = fmaxf(ds, de);
    ds = __fmul_rn(__fsub_rn(ly, o.y), inv.y);
    de = __fmul_rn(__fsub_rn(hy, o.y), inv.y);
    mn = fmaxf(mn, fminf(ds, de));
    mx = fminf(mx, fmaxf(ds, de));
    ds = __fmul_rn(__fsub_rn(lz, o.z), inv.z);
    de = __fmul_rn(__fsub_rn(hz, o.z), inv.z);
    mn = fmaxf(mn, fminf(ds, de));
    mx = fminf(mx, fmaxf(ds, de));
    if (mn > __fadd_rn(mx, kEps)) return false;
    if (front && mx < -kEps) return false;  // entirely behind the origin (front_only scenes)
    return mn != FLT_MAX;
}

// One edge condition of Triangle::containsVertex (Triangle.impl.h:292-302):
//     rn(rn(X / rn(sqrt(P))) + S) >= rn(Y / rn(sqrt(Q)))
// with X = e.px, P = px.px, Y = -(e.f), Q = f.f (all exactly rounded dot products).
// Decided first with rsqrtf (documented max error 2 ulp): the fast left and right sides differ from
// the exactly rounded ones by at most ~3 ulp each, so a difference D outside the margin
// M = 2^-19 (|L| + |R| + S) (about 16 ulp) has the same sign as the exact difference; inside the
// margin, or for inf/NaN operands, the exact IEEE expression is evaluated.  Results are therefore
// bit-identical to the reference's host arithmetic while the common case avoids two IEEE divisions
// and two IEEE square roots.
__device__ __forceinline__ bool edge_ok(f3 e, f3 px, f3 f) {
    const float S = 32 * kEps;
    const float X = xdot(e, px), P = xdot(px, px), Y = -xdot(e, f), Q = xdot(f, f);
    const float Lf = __fadd_rn(__fmul_rn(X, rsqrtf(P)), S);
    const float Rf = __fmul_rn(Y, rsqrtf(Q));
    const float D = __fsub_rn(Lf, Rf);
    const float M = 1.9073486328125e-06f * (fabsf(Lf) + fabsf(Rf) + S);
    if (D > M) return true;
    if (D < -M) return false;
    return __fadd_rn(__fdiv_rn(X, __fsqrt_rn(P)), S) >= __fdiv_rn(Y, __fsqrt_rn(Q));
}

// Triangle::containsVertex (Triangle.impl.h:283-302)
__device__ __forceinline__ bool contains_vertex(f3 a, f3 b, f3 c, f3 p) {
    if (xeq(a, b) || xeq(b, c) || xeq(c, a)) return false;
    if (xeq(p, a) || xeq(p, b) || xeq(p, c)) return true;
    f3 ab = xsub(b, a), bc = xsub(c, b), ca = xsub(a, c);
    if (!edge_ok(ab, xsub(p, a), ca)) return false;
    if (!edge_ok(bc, xsub(p, b), ab)) return false;
    return edge_ok(ca, xsub(p, c), bc);
}

// Triangle::cast (Triangle.impl.h:334-348), with the caller's strict-min and validator checks
// (castInLeaf, Octree.impl.cuh:596-603) moved ahead of the containment test: a triangle whose
// distance is not below `best`, or that is the ignored object, cannot change the leaf's result,
// so skipping its containment test leaves every result unchanged.
__device__ __forceinline__ bool tri_cast_better(f3 a, f3 b, f3 c, int id, f3 o, f3 d, bool clip, int ignore, float best,
                                                float &dist, f3 &hp) {
    f3 n = xcross(xsub(b, a), xsub(c, a));
    float dp = xdot(xsub(a, o), n);
    if (clip && (dp < -kEps)) return false;
    float dirp = xdot(d, n);
    if (__fmul_rn(dp, dirp) <= 0.0f) return false;
    float distance = __fdiv_rn(dp, dirp);
    if (!(distance < best) || id == ignore) return false;
    f3 hv = xadd(o, xmul(d, distance));
    if (!contains_vertex(a, b, c, hv)) return false;
    dist = distance;
    hp = hv;
    return true;
}

struct Hit {
    int tri;     // -1 = miss
    float t;     // in units of |d|
    f3 p;        // hit point o + d * t (exactly as the reference computes it)
};

// castInLeaf (Octree.impl.cuh:584-612): strict-min distance over the leaf list (ties keep the
// first), `ignore` = validateNotSameAsObject, accept only if the hit point is inside the leaf box.
__device__ __forceinline__ bool cast_leaf(const Scene &S, int first, int count, float lx, float ly, float lz, float hx,
                                          float hy, float hz, f3 o, f3 d, bool clip, int ignore, Hit &h, int &ntri) {
    if (count <= 0) return false;
    float best = FLT_MAX;
    f3 bp = mkf3(0.f, 0.f, 0.f);
    int bi = -1;
    const float4 *lt = S.leaf_tris + 3 * (size_t)first;
    for (int r = 0; r < count; r++) {
        float4 A = __ldg(lt + 3 * r), B = __ldg(lt + 3 * r + 1), C = __ldg(lt + 3 * r + 2);
        int id = __float_as_int(A.w);
        float dist;
        f3 hp;
        ntri++;
        if (tri_cast_better(f3of(A), f3of(B), f3of(C), id, o, d, clip, ignore, best, dist, hp)) {
            best = dist;
            bp = hp;
            bi = id;
        }
    }
    if (best != FLT_MAX && bp.x >= lx && bp.y >= ly && bp.z >= lz && bp.x <= hx && bp.y <= hy && bp.z <= hz) {
        h.tri = bi;
        h.t = best;
        h.p = bp;
        return true;
    }
    return false;
}

// Tests the 8 children of a group; bit k of the result = child (order ^ k) is hit.  The slab tests
// of the 8 children run plane by plane on the plane layout (x entry/exit of all children, then y,
// then z), which keeps 16 running values instead of 48 coordinates live; each child's operations are
// those of slab_hit in the same order.  Bit c of the octant-order mask then moves to c ^ order, so
// results and counts equal a test in visit order.
// Two consecutive float4 (32 bytes, 32-byte aligned) in one 256-bit read-only load (sm_100 and
// later): a node record.  Half the load instructions of two 128-bit loads, for the same bytes.  (The
// child-box planes keep 128-bit loads: 256-bit destinations raised the traversal's spills from 20 to
// 154 bytes at its 80-register budget.)
__device__ __forceinline__ void ldg2(const float4 *p, float4 &a, float4 &b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ void slab_planes(const float4 *g, int plane, float oc, float ic, float *mn, float *mx, bool first) {
    const float4 l0 = __ldg(g + 2 * plane), l1 = __ldg(g + 2 * plane + 1);
    const float4 h0 = __ldg(g + 6 + 2 * plane), h1 = __ldg(g + 6 + 2 * plane + 1);
    const float lo[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
    const float hi[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float ds = __fmul_rn(__fsub_rn(lo[c], oc), ic);
        const float de = __fmul_rn(__fsub_rn(hi[c], oc), ic);
        if (first) {
            mn[c] = fminf(ds, de);
            mx[c] = fmaxf(ds, de);
        } else {
            mn[c] = fmaxf(mn[c], fminf(ds, de));
            mx[c] = fminf(mx[c], fmaxf(ds, de));
        }
    }
}

__device__ __forceinline__ unsigned test_group(const float4 *gbox, int group, int order, f3 o, f3 inv, bool front) {
    const float4 *g = gbox + 12 * (size_t)group;
    float mn[8], mx[8];
    slab_planes(g, 0, o.x, inv.x, mn, mx, true);
    slab_planes(g, 1, o.y, inv.y, mn, mx, false);
    slab_planes(g, 2, o.z, inv.z, mn, mx, false);
    unsigned m = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const bool hit = !(mn[c] > __fadd_rn(mx[c], kEps)) && !(front && mx[c] < -kEps) && mn[c] != FLT_MAX;
        m |= (hit ? 1u : 0u) << c;
    }
    if (order & 1) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (order & 2) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (order & 4) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    return m;
}

// Octree::cast (Octree.impl.cuh:174-212).  Visits children in the reference's sign order
// (canonicalOrder ^ k); the 8 slab tests of a group are done up front (they are pure), which
// visits exactly the same leaves in the same order.  With COUNT, nbox receives the number of
// child-box tests the reference's sequential scan performs (it stops scanning a group when a hit
// is returned below it) plus the root test, and ntri the triangle tests.
// Traversal stack entry: group << shift | (COUNT: child position taken << 8) | remaining hit mask.
// The position is only needed to correct the box-test count, so the counting kernels keep 21 bits
// of group index (2^24 nodes) and the others 24 (2^27 nodes, room for a batch arena).
template <bool COUNT>
__host__ __device__ constexpr int group_shift() { return COUNT ? 11 : 8; }

template <bool COUNT>
__device__ __forceinline__ bool cast_closest(const Scene &S, f3 o, f3 d, bool clip, int ignore, Hit &h, int &nbox,
                                             int &ntri) {
    h.tri = -1;
    h.t = FLT_MAX;
    f3 inv = mkf3(__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z));
    if (S.root_child < 0)
        return cast_leaf(S, S.root_leaf_first, S.root_leaf_count, S.root_lo[0], S.root_lo[1], S.root_lo[2], S.root_hi[0],
                         S.root_hi[1], S.root_hi[2], o, d, clip, ignore, h, ntri);
    if (COUNT) nbox++;
    const bool front = !COUNT || S.front_only != 0;
    const float4 *G = front ? S.gbox : S.gbox_ref;
    if (!slab_hit(S.root_lo[0], S.root_lo[1], S.root_lo[2], S.root_hi[0], S.root_hi[1], S.root_hi[2], o, inv, front)) return false;
    const int order = (d.z < 0 ? 1 : 0) + (d.y < 0 ? 2 : 0) + (d.x < 0 ? 4 : 0);
    constexpr int GS = group_shift<COUNT>();
    uint32_t stack[kStack];
    int sp = 0;
    uint32_t cur = ((uint32_t)S.root_child << GS) | test_group(G, S.root_child, order, o, inv, front);
    if (COUNT) nbox += 8;
    for (;;) {
        uint32_t m = cur & 0xFFu;
        if (m == 0) {
            if (sp == 0) return false;
            cur = stack[--sp];
            continue;
        }
        int k = __ffs(m) - 1;
        cur &= ~(1u << k);
        int group = (int)(cur >> GS);
        int node = group * 8 + (order ^ k);
        float4 lo, hi;
        ldg2(S.nodes + 2 * (size_t)node, lo, hi);
        int w = __float_as_int(lo.w);
        if (w < 0) {
            if (cast_leaf(S, ~w, __float_as_int(hi.w), lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, o, d, clip, ignore, h, ntri)) {
                if (COUNT) {
                    nbox -= 7 - k;
                    for (int s = 0; s < sp; s++) nbox -= 7 - (int)((stack[s] >> 8) & 7u);
                }
                return true;
            }
        } else {
            if (sp >= kStack) return false;  // unreachable for trees of depth <= 24
            stack[sp++] = COUNT ? ((cur & ~(7u << 8)) | ((uint32_t)k << 8)) : cur;
            cur = ((uint32_t)(w >> 3) << GS) | test_group(G, w >> 3, order, o, inv, front);
            if (COUNT) nbox += 8;
        }
    }
}

// ---- counter-based random numbers ----------------------------------------------------------
// u32 = H(H(key + 0x9E3779B9 * (bounce * 128 + dim + 1))), key = H(H(H(seed ^ 0x2545F491) ^ pixel) + sample),
// H = lowbias32 (C. Wellons' public-domain integer hash).  Float = (u >> 8) * 2^-24 in [0, 1).
__host__ __device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
__host__ __device__ __forceinline__ uint32_t path_key(uint32_t seed, uint32_t pixel, uint32_t sample) {
    return hash32(hash32(hash32(seed ^ 0x2545F491U) ^ pixel) + sample);
}
__device__ __forceinline__ float rnd(uint32_t key, uint32_t bounce, uint32_t dim) {
    uint32_t u = hash32(hash32(key + 0x9E3779B9U * (bounce * 128U + dim + 1U)));
    return (float)(u >> 8) * (1.0f / 16777216.0f);
}
constexpr uint32_t kLensBounce = 1023;

}  // namespace drd
