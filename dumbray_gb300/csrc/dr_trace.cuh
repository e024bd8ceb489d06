// dr_trace.cuh - persistent, warp-refilled octree traversal for ray batches.
//
// Each lane traces one ray at a time with exactly the visit order and leaf semantics of
// Octree::cast (Octree.impl.cuh:174-212, castInLeaf :584-612), so results are identical to
// cast_closest().  What changes is the scheduling across the 32 lanes of a warp:
//   * one unit of work per lane per loop iteration: either one traversal step (stack pops plus at
//     most one 8-child group test, or entering a leaf) or one triangle test.  A lane never waits
//     for another lane's whole leaf or whole descent; per-ray costs range over three orders of
//     magnitude on displaced meshes (p99 ~1,700 triangle tests against a mean of ~120);
//   * leaf work is shared by the whole warp: the pending (ray, triangle) tests of all lanes that hold
//     a leaf are numbered with a warp prefix sum and handed out 64 per round, two per lane; the
//     tester reads the owner's ray through shuffles and posts (distance, list position) to the
//     owner's slot with a 64-bit atomicMin, so the owner keeps the smallest distance and, among
//     equal distances, the earliest triangle in list order - exactly castInLeaf's strict-min scan;
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
    const bool front = !COUNT || S.front_only != 0;
    if (slab_hit(S.root_lo[0], S.root_lo[1], S.root_lo[2], S.root_hi[0], S.root_hi[1], S.root_hi[2], L.o, L.inv, front)) {
        L.cur = ((uint32_t)S.root_child << group_shift<COUNT>()) |
                test_group(front ? S.gbox : S.gbox_ref, S.root_child, L.order, L.o, L.inv, front);
        if (COUNT) L.nb += 8;
    }
    return kTrav;
}

// Loads entry i of the source into the lane and starts its ray; kIdle when the source has nothing
// to trace for it.  Also serves a ray the source rewrote in place (a photon continuing past a
// blocker): the lane starts it at once, without going back to the warp's chunk.
template <bool COUNT, bool MULTI, class Source>
__device__ __forceinline__ int restart(const Scene &S, Source &src, int i, LaneRay &L) {
    int ign, job;
    if (!src.load(i, L.o, L.d, ign, job)) return kIdle;
    L.ignore = ign;
    return lane_start<COUNT>(MULTI ? src.scene(job) : S, L);
}

// Per-warp shared scratch of the cooperative leaf rounds.
struct WarpLeafSlots {
    unsigned long long key[32];
    int incl[32];
};

// Source interface:
//   bool next(int &begin, int &end)           warp-uniform; false when no work is left
//   bool load(int i, f3 &o, f3 &d, int &ignore, int &job)   false: entry i needs no cast (done)
//   const Scene &scene(int job)               the scene of a job (MULTI only)
//   bool clip(int job)                        backface culling of a job (MULTI = false: job 0 for all)
//   bool store(int i, const Hit &h, int nbox, int ntri)   true: ray i was rewritten (load() now
//                                             gives its next cast) and the lane traces it at once
//   static constexpr float kOccludeBelow      > 0: visibility-only rays (any hit nearer than this
//                                             settles them); 0: closest hit
// MULTI = false: every ray belongs to scene `S`.  MULTI = true: rays of different scenes share the
// warp; their trees live in one batch arena (S.nodes / S.leaf_tris are the arena's), so a lane only
// takes its scene's root (bounds, child group or root leaf) when it starts a ray.  Backface culling
// is uniform over a wave in both cases.
template <bool COUNT, bool MULTI, class Source>
// steps_per_round: traversal steps a lane may take between two cooperative leaf rounds while it
// stays in inner nodes; more means fewer per-round ballots and prefix sums, but lanes that reached a
// leaf wait longer (measured: 2 pays on physical-tree scenes, whose leaves are small; 1 elsewhere).
__device__ __forceinline__ void trace_persistent(const Scene &S, Source &src, uint32_t *stack, WarpLeafSlots &ws,
                                                 int steps_per_round = 1) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    int c_next = 0, c_end = 0;
    bool drained = false;
    int cur_i = -1;
    int mode = kIdle;
    constexpr int GS = group_shift<COUNT>();
    const bool clip = src.clip(0);
    const bool front = !COUNT || S.front_only != 0;   // uniform: one scene, or one arena of a batch
    // group-test planes: refitted, except for counting on reference-padding scenes (their counts are
    // the reference's)
    const float4 *G = front ? S.gbox : S.gbox_ref;
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
                    mode = restart<COUNT, MULTI>(S, src, cur_i, L);
                }
                c_next += min(avail, __popc(want));
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, mode != kIdle) == 0u) {
            if (drained) break;
            continue;
        }
#pragma unroll 1
        for (int step = 0; step < steps_per_round; step++) {
        if (mode != kTrav) break;
        {
            // ---- one traversal step: pop empty frames, then take one child
            while ((L.cur & 0xFFu) == 0u && L.sp > 0) L.cur = stack[--L.sp];
            uint32_t m = L.cur & 0xFFu;
            if (m == 0u) {
                Hit h;
                h.tri = -1;
                h.t = FLT_MAX;
                mode = src.store(cur_i, h, L.nb, L.nt) ? restart<COUNT, MULTI>(S, src, cur_i, L) : kIdle;
            } else {
                int k = __ffs(m) - 1;
                L.cur &= ~(1u << k);
                int node = (int)(L.cur >> GS) * 8 + (L.order ^ k);
                float4 lo, hi;
                ldg2(S.nodes + 2 * (size_t)node, lo, hi);
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
                    stack[L.sp++] = COUNT ? ((L.cur & ~(7u << 8)) | ((uint32_t)k << 8)) : L.cur;
                    L.cur = ((uint32_t)(w >> 3) << GS) | test_group(G, w >> 3, L.order, L.o, L.inv, front);
                    if (COUNT) L.nb += 8;
                } else {  // unreachable for depth <= 24: finish as a miss rather than overflow
                    L.cur = 0;
                    L.sp = 0;
                }
            }
        }
        }
        // ---- one cooperative round of leaf triangle tests (castInLeaf)
        int pending = (mode == kLeaf) ? (L.r_end - L.r) : 0;
        int incl = pending;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if ((int)lane >= off) incl += v;
        }
        const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        if (total > 0) {
            ws.incl[lane] = incl;
            ws.key[lane] = ~0ull;
            __syncwarp();
            // tasks `lane` and `lane + 32` of this round; task t belongs to the first lane whose
            // inclusive count exceeds t.  Both triangles are loaded before either is tested.
            const int t0 = (int)lane, t1 = (int)lane + 32;
            int own0 = (int)lane, own1 = (int)lane;
            if (t0 < total) {
                own0 = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (ws.incl[own0 + step - 1] <= t0) own0 += step;
            }
            if (t1 < total) {
                own1 = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (ws.incl[own1 + step - 1] <= t1) own1 += step;
            }
            const int excl0 = ws.incl[own0] - __shfl_sync(0xFFFFFFFFu, pending, own0);
            const int excl1 = ws.incl[own1] - __shfl_sync(0xFFFFFFFFu, pending, own1);
            const int r0 = __shfl_sync(0xFFFFFFFFu, L.r, own0), r1 = __shfl_sync(0xFFFFFFFFu, L.r, own1);
            const int pos0 = r0 + (t0 - excl0), pos1 = r1 + (t1 - excl1);
            float4 A0, B0, C0, A1, B1, C1;
            if (t0 < total) {
                const float4 *lt = S.leaf_tris + 3 * (size_t)pos0;
                A0 = __ldg(lt); B0 = __ldg(lt + 1); C0 = __ldg(lt + 2);
            }
            if (t1 < total) {
                const float4 *lt = S.leaf_tris + 3 * (size_t)pos1;
                A1 = __ldg(lt); B1 = __ldg(lt + 1); C1 = __ldg(lt + 2);
            }
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int own = q ? own1 : own0;
                const float ox = __shfl_sync(0xFFFFFFFFu, L.o.x, own), oy = __shfl_sync(0xFFFFFFFFu, L.o.y, own),
                            oz = __shfl_sync(0xFFFFFFFFu, L.o.z, own);
                const float dx = __shfl_sync(0xFFFFFFFFu, L.d.x, own), dy = __shfl_sync(0xFFFFFFFFu, L.d.y, own),
                            dz = __shfl_sync(0xFFFFFFFFu, L.d.z, own);
                const int ign = __shfl_sync(0xFFFFFFFFu, L.ignore, own);
                const float obest = __shfl_sync(0xFFFFFFFFu, L.best, own);
                if ((q ? t1 : t0) < total) {
                    const float4 A = q ? A1 : A0, B = q ? B1 : B0, C = q ? C1 : C0;
                    float dist;
                    f3 hp;
                    if (tri_cast_better(f3of(A), f3of(B), f3of(C), __float_as_int(A.w), mkf3(ox, oy, oz), mkf3(dx, dy, dz),
                                        clip, ign, obest, dist, hp))
                        atomicMin(&ws.key[own], ((unsigned long long)__float_as_uint(dist) << 32) | (unsigned)(q ? pos1 : pos0));
                }
            }
            __syncwarp();
            if (mode == kLeaf) {
                const int excl = incl - pending;
                const int done = max(0, min(pending, 64 - excl));
                if (COUNT) L.nt += done;
                L.r += done;
                const unsigned long long k = ws.key[lane];
                if (k != ~0ull) {
                    const float dist = __uint_as_float((unsigned)(k >> 32));
                    const int pos = (int)(k & 0xFFFFFFFFull);
                    L.best = dist;
                    L.bi = __float_as_int(__ldg(S.leaf_tris + 3 * (size_t)pos).w);
                    L.bp = xadd(L.o, xmul(L.d, dist));
                }
            }
            __syncwarp();
        }
        if (mode == kLeaf && L.r >= L.r_end) {
            // occlusion sources end a ray at the first leaf holding a hit nearer than their limit, even
            // one whose point lies in a later leaf: that hit's own leaf would end the ray there anyway
            const bool occluded = Source::kOccludeBelow > 0.0f && L.best < Source::kOccludeBelow;
            if (L.best != FLT_MAX && (occluded || (L.bp.x >= L.lx && L.bp.y >= L.ly && L.bp.z >= L.lz && L.bp.x <= L.hx &&
                                                   L.bp.y <= L.hy && L.bp.z <= L.hz))) {
                if (COUNT) {
                    L.nb -= 7 - L.kleaf;
                    for (int s = 0; s < L.sp; s++) L.nb -= 7 - (int)((stack[s] >> 8) & 7u);
                }
                Hit h;
                h.tri = L.bi;
                h.t = L.best;
                h.p = L.bp;
                mode = src.store(cur_i, h, L.nb, L.nt) ? restart<COUNT, MULTI>(S, src, cur_i, L) : kIdle;
            } else {
                mode = kTrav;
            }
        }
    }
}

}  // namespace drd
