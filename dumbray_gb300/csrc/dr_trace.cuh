// dr_trace.cuh - persistent, warp-refilled octree traversal for ray batches.
//
// Each lane traces one ray at a time with exactly the visit order and leaf semantics of
// Octree::cast (Octree.impl.cuh:174-212, castInLeaf :584-612), so results are identical to
// cast_closest().  What changes is the scheduling across the 32 lanes of a warp:
//   * one unit of work per lane per loop iteration: either one traversal step (stack pops plus at
//     most one 8-child group test, or entering a leaf) or one triangle test.  A lane never waits
//     for another lane's whole leaf or whole descent; per-ray costs range over three orders of
//     magnitude on displaced meshes (p99 ~1,700 triangle tests against a mean of ~120);
//   * a lane whose ray is finished takes the next ray of the warp's current chunk at once.  Chunks
//     are handed out by the caller's Source (an atomic counter for queues whose size is only known
//     on the device, a fixed range for plain batches).
#pragma once
#include "dr_device.cuh"

namespace drd {

constexpr int kChunk = 256;

enum : int { kIdle = 0, kTrav = 1, kLeaf = 2 };

struct LaneRay {
    f3 o, d, inv;
    int order, ignore;
    uint32_t cur;
    int sp;
    int r, r_end;
    float lx, ly, lz, hx, hy, hz;
    float best;
    f3 bp;
    int bi;
    int kleaf;
    int nb, nt;
};

// Starts a ray: root leaf, root miss, or the root's children tested (Octree.impl.cuh:175-190).
template <bool COUNT>
__device__ __forceinline__ int lane_start(const Scene &S, LaneRay &L) {
    L.inv = mkf3(__fdiv_rn(1.0f, L.d.x), __fdiv_rn(1.0f, L.d.y), __fdiv_rn(1.0f, L.d.z));
    L.order = (L.d.z < 0 ? 1 : 0) + (L.d.y < 0 ? 2 : 0) + (L.d.x < 0 ? 4 : 0);
    L.sp = 0;
    L.cur = 0;
    L.nb = 0;
    L.nt = 0;
    L.kleaf = 0;
    if (S.root_child < 0) {
        L.r = S.root_leaf_first;
        L.r_end = S.root_leaf_first + S.root_leaf_count;
        L.lx = S.root_lo[0]; L.ly = S.root_lo[1]; L.lz = S.root_lo[2];
        L.hx = S.root_hi[0]; L.hy = S.root_hi[1]; L.hz = S.root_hi[2];
        L.best = FLT_MAX;
        L.bi = -1;
        L.kleaf = 7;  // no group scan to correct for a root leaf
        return kLeaf;
    }
    if (COUNT) L.nb++;
    if (slab_hit(S.root_lo[0], S.root_lo[1], S.root_lo[2], S.root_hi[0], S.root_hi[1], S.root_hi[2], L.o, L.inv)) {
        L.cur = test_group(S, 0, L.order, L.o, L.inv);
        if (COUNT) L.nb += 8;
    }
    return kTrav;
}

// Source interface:
//   bool next(int &begin, int &end)           warp-uniform; false when no work is left
//   void load(int i, f3 &o, f3 &d, int &ignore)
//   void store(int i, const Hit &h, int nbox, int ntri)
template <bool COUNT, class Source>
__device__ __forceinline__ void trace_persistent(const Scene &S, bool clip, Source &src, uint32_t *stack) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    int c_next = 0, c_end = 0;
    bool drained = false;
    int cur_i = -1;
    int mode = kIdle;
    LaneRay L;
    L.r = 0;
    L.r_end = 0;
    L.sp = 0;
    L.cur = 0;
    L.best = FLT_MAX;
    L.bi = -1;
    for (;;) {
        // ---- refill idle lanes from the warp's chunk (warp-uniform control flow)
        unsigned want = __ballot_sync(0xFFFFFFFFu, mode == kIdle);
        if (want != 0u && !drained) {
            if (c_next >= c_end && !src.next(c_next, c_end)) drained = true;
            if (!drained) {
                int avail = c_end - c_next;
                int rank = __popc(want & lt_mask);
                if (mode == kIdle && rank < avail) {
                    cur_i = c_next + rank;
                    int ign;
                    src.load(cur_i, L.o, L.d, ign);
                    L.ignore = ign;
                    mode = lane_start<COUNT>(S, L);
                }
                c_next += min(avail, __popc(want));
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, mode != kIdle) == 0u) {
            if (drained) break;
            continue;
        }
        if (mode == kTrav) {
            // ---- one traversal step: pop empty frames, then take one child
            while ((L.cur & 0xFFu) == 0u && L.sp > 0) L.cur = stack[--L.sp];
            uint32_t m = L.cur & 0xFFu;
            if (m == 0u) {
                Hit h;
                h.tri = -1;
                h.t = FLT_MAX;
                src.store(cur_i, h, L.nb, L.nt);
                mode = kIdle;
            } else {
                int k = __ffs(m) - 1;
                L.cur &= ~(1u << k);
                int node = (int)(L.cur >> 11) * 8 + (L.order ^ k);
                float4 lo = __ldg(S.nodes + 2 * (size_t)node), hi = __ldg(S.nodes + 2 * (size_t)node + 1);
                int w = __float_as_int(lo.w);
                if (w < 0) {
                    L.r = ~w;
                    L.r_end = ~w + __float_as_int(hi.w);
                    L.lx = lo.x; L.ly = lo.y; L.lz = lo.z;
                    L.hx = hi.x; L.hy = hi.y; L.hz = hi.z;
                    L.best = FLT_MAX;
                    L.bi = -1;
                    L.kleaf = k;
                    mode = kLeaf;
                } else if (L.sp < kStack) {
                    stack[L.sp++] = (L.cur & ~(7u << 8)) | ((uint32_t)k << 8);
                    L.cur = ((uint32_t)(w >> 3) << 11) | test_group(S, w >> 3, L.order, L.o, L.inv);
                    if (COUNT) L.nb += 8;
                } else {  // unreachable for depth <= 24: finish as a miss rather than overflow
                    L.cur = 0;
                    L.sp = 0;
                }
            }
        } else if (mode == kLeaf) {
            // ---- one triangle test of the current leaf (castInLeaf)
            if (L.r < L.r_end) {
                const float4 *lt = S.leaf_tris + 3 * (size_t)L.r;
                float4 A = __ldg(lt), B = __ldg(lt + 1), C = __ldg(lt + 2);
                float dist;
                f3 hp;
                if (COUNT) L.nt++;
                if (tri_cast_better(f3of(A), f3of(B), f3of(C), __float_as_int(A.w), L.o, L.d, clip, L.ignore, L.best, dist, hp)) {
                    L.best = dist;
                    L.bp = hp;
                    L.bi = __float_as_int(A.w);
                }
                L.r++;
            }
            if (L.r >= L.r_end) {
                if (L.best != FLT_MAX && L.bp.x >= L.lx && L.bp.y >= L.ly && L.bp.z >= L.lz && L.bp.x <= L.hx &&
                    L.bp.y <= L.hy && L.bp.z <= L.hz) {
                    if (COUNT) {
                        L.nb -= 7 - L.kleaf;
                        for (int s = 0; s < L.sp; s++) L.nb -= 7 - (int)((stack[s] >> 8) & 7u);
                    }
                    Hit h;
                    h.tri = L.bi;
                    h.t = L.best;
                    h.p = L.bp;
                    src.store(cur_i, h, L.nb, L.nt);
                    mode = kIdle;
                } else {
                    mode = kTrav;
                }
            }
        }
    }
}

}  // namespace drd
