// dr_kernels.cu - sm_103a kernels of the GB300 DumbRay hot path.
//
//   k_cast            ray batch -> closest hit (Octree::cast, Octree.impl.cuh:174-212)
//   k_camera          per path: lens sample -> ray queue            (Lense::getPixelSamples)
//   k_trace           ray queue -> hit records                       (Octree::cast)
//   k_shade_ref       DumbRenderer layer step (DumbRenderer.cu:249-443) as one forward path step:
//                     indirect request, light photons -> shadow queue, next ray -> next queue
//   k_shadow_ref      light -> point visibility, first cast of every photon (DumbRenderer.cu:361-428)
//   k_photon_chain    photons stopped by a blocker: the reference's transparency re-casts
//   k_shade_phys      physical path step (emission + MIS, NEE -> shadow queue, BSDF sample);
//                     in the adjoint pass it also scatters gradients of emission hits
//   k_shadow_phys     point -> light visibility; in the adjoint pass it marks the visible records
//   k_adj_shadow      adjoint pass: gradients of the visible NEE contributions
//   k_resolve         accumulators -> BlockBasedFrameBuffer<8,16> set / blend (BlockBasedFrameBuffer.impl.cuh:149-156)
//
// Wavefront design: queues are structure-of-arrays of float4/int4 records in HBM; work is pulled by
// persistent warps (shading: blocks) through one atomic per warp (block); outputs are compacted with
// ballots and one atomic per warp (block; rays grouped by direction octant).  Queue counts live in
// a device control block, so a whole wave is a fixed launch sequence with no host synchronisation
// (and can be captured in a CUDA graph).  Every path record carries the index of its render job, so
// the paths of many scenes can share a wave (batches).
#include <algorithm>
#include <atomic>
#include "dr_kernels.h"
#include "dr_shading.cuh"
#include "dr_trace.cuh"

#include <cstdio>

namespace drd {

using drk::Item;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated slot allocation: every lane of the warp must call this together.
__device__ __forceinline__ int warp_alloc(int *counter, bool want) {
    unsigned ballot = __ballot_sync(0xFFFFFFFFu, want);
    if (ballot == 0) return -1;
    int leader = __ffs(ballot) - 1;
    int base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return want ? base + __popc(ballot & ((1u << lane_id()) - 1u)) : -1;
}

// Block-wide steps of the shading kernels (kShadeThreads threads, every thread calls both
// together): fetch the block's next kShadeThreads queue entries, then allocate the children's
// slots in the next queue with the block's children grouped by direction octant.  The block's
// paths are neighbouring pixels of one sample, so a warp of the next trace gets rays leaving
// nearby points into one octant, which descend the octree along the same nodes.
constexpr int kShadeThreads = 256;
struct ShadeBlockShared {
    int base, out;
    int cnt[kShadeThreads / 32][8];  // [warp][octant]: counts, then exclusive offsets
};
__device__ __forceinline__ int block_fetch(int *counter, ShadeBlockShared &sh) {
    if (threadIdx.x == 0) sh.base = atomicAdd(counter, kShadeThreads);
    __syncthreads();
    return sh.base;
}
__device__ __forceinline__ int block_alloc_by_octant(int *counter, bool want, f3 dir, ShadeBlockShared &sh) {
    const int oct = (dir.x < 0.0f) | ((dir.y < 0.0f) << 1) | ((dir.z < 0.0f) << 2);
    const int wid = (int)(threadIdx.x >> 5);
    unsigned mine = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const unsigned m = __ballot_sync(0xFFFFFFFFu, want && oct == k);
        if (want && oct == k) mine = m;
        if (lane_id() == 0) sh.cnt[wid][k] = __popc(m);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int total = 0;
        for (int k = 0; k < 8; k++)
            for (int v = 0; v < kShadeThreads / 32; v++) {
                const int c = sh.cnt[v][k];
                sh.cnt[v][k] = total;
                total += c;
            }
        sh.out = total ? atomicAdd(counter, total) : 0;
    }
    __syncthreads();
    return want ? sh.out + sh.cnt[wid][oct] + __popc(mine & ((1u << lane_id()) - 1u)) : -1;
}

// Warp-level work fetch from a dynamic counter; returns the base index (warp-uniform).
__device__ __forceinline__ int warp_fetch(int *counter) {
    int base = 0;
    if (lane_id() == 0) base = atomicAdd(counter, 32);
    return __shfl_sync(0xFFFFFFFFu, base, 0);
}

// Chunked work fetch from a device counter (warp-uniform).  The chunk shrinks with the queue:
// about 4 chunks per resident warp (152 SMs x 24 warps), between 32 and kChunk rays, so short
// queues (late bounces, shadow queues) still spread over every resident warp.
__device__ __forceinline__ int chunk_for(int n) { return max(32, min(kChunk, (n / (152 * 24 * 4)) & ~31)); }
__device__ __forceinline__ bool fetch_chunk(int *counter, int n, int chunk, int &b, int &e) {
    int base = 0;
    if ((threadIdx.x & 31u) == 0) base = atomicAdd(counter, chunk);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (base >= n) return false;
    b = base;
    e = min(base + chunk, n);
    return true;
}

__device__ __forceinline__ void count_add64(unsigned long long *c, long long rays, long long nb, long long nt) {
    for (int off = 16; off > 0; off >>= 1) {
        rays += __shfl_xor_sync(0xFFFFFFFFu, rays, off);
        nb += __shfl_xor_sync(0xFFFFFFFFu, nb, off);
        nt += __shfl_xor_sync(0xFFFFFFFFu, nt, off);
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(c, (unsigned long long)rays);
        atomicAdd(c + 1, (unsigned long long)nb);
        atomicAdd(c + 2, (unsigned long long)nt);
    }
}

__device__ __forceinline__ void accum_add(float *acc, int slot, c3 c) {
    if (c.r != 0.0f) atomicAdd(acc + 4 * slot, c.r);
    if (c.g != 0.0f) atomicAdd(acc + 4 * slot + 1, c.g);
    if (c.b != 0.0f) atomicAdd(acc + 4 * slot + 2, c.b);
}

// ---------------------------------------------------------------------------------------------
// dr_cast: warp w of the grid owns rays [w * kChunk, (w + 1) * kChunk) of one scene.
struct BatchSource {
    static constexpr float kOccludeBelow = 0.0f;
    const float *o, *d;
    const int *ignore;
    int *hit_tri, *nbox, *ntri;
    float *hit_t;
    int n;
    bool given, cull;
    const Scene *scene0;  // unused: single-scene source
    __device__ __forceinline__ bool next(int &b, int &e) {
        if (given) return false;
        given = true;
        int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
        b = w * kChunk;
        e = min(b + kChunk, n);
        return b < n;
    }
    __device__ __forceinline__ bool load(int i, f3 &ro, f3 &rd, int &ign, int &job) {
        ro = mkf3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
        rd = mkf3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
        ign = ignore ? ignore[i] : -1;
        job = 0;
        return true;
    }
    // single-scene source: never asked for a per-job scene (MULTI = false)
    __device__ __forceinline__ const Scene &scene(int) { return *scene0; }
    __device__ __forceinline__ bool clip(int) { return cull; }
    __device__ __forceinline__ bool store(int i, const Hit &h, int nb, int nt) {
        hit_tri[i] = h.tri;
        hit_t[i] = h.tri >= 0 ? h.t : FLT_MAX;
        if (nbox) {
            nbox[i] = nb;
            ntri[i] = nt;
        }
        return false;
    }
};

template <bool COUNT>
__global__ void __launch_bounds__(128) k_cast(Scene S, const float *__restrict__ o, const float *__restrict__ d,
                                              const int *__restrict__ ignore, int n, int clip, int *__restrict__ hit_tri,
                                              float *__restrict__ hit_t, int *__restrict__ nbox, int *__restrict__ ntri) {
    uint32_t stack[kStack];
    __shared__ WarpLeafSlots slots[4];
    BatchSource src{o, d, ignore, hit_tri, COUNT ? nbox : nullptr, COUNT ? ntri : nullptr, hit_t, n, false, clip != 0, &S};
    trace_persistent<COUNT, false>(S, src, stack, slots[threadIdx.x >> 5]);
}

// ---------------------------------------------------------------------------------------------
// Wave control block (int slots, zeroed at the start of every wave).
struct Ctrl {
    int ray_count[kMaxBounceSlots];
    int shadow_count[kMaxBounceSlots];
    int fetch_trace[kMaxBounceSlots];
    int fetch_shade[kMaxBounceSlots];
    int fetch_shadow[kMaxBounceSlots];
    int blocked_count[kMaxBounceSlots];   // reference photons stopped by a blocker at bounce b and
    int fetch_chain[kMaxBounceSlots];     // left in place (the carry region was full)
    int carry_count;                      // blocked reference photons moved to the carry region
    int fetch_carry;
    int fetch_camera;
    int error;
};

// Ray queue record (64 B, 4 x 16 B SoA planes):
//   p0 = {o.xyz, accumulator slot}   p1 = {d.xyz, sample index}   p2 = {throughput.rgb, prev pdf}
//   p3 = {prev triangle, flags (bit 0 = prev vertex delta; bits 1.. = path index in the wave), pixel id, job}
struct Queue {
    float4 *p0, *p1, *p2;
    int4 *p3;
};
// Hit record: {tri, t}
// Shadow record (80 B): s0 = {origin.xyz, accumulator slot}, s1 = {dir.xyz, target / light tri},
//   s2 = {target point.xyz, ignore tri}, s3 = {light colour rgb | adjoint: path index, vertex, -}, s4 = {contribution rgb, job}
struct ShadowQ {
    float4 *s0, *s1, *s2, *s3, *s4;
};

struct WaveArgs {
    Item inl;
    const Item *items;
    int n_items;
    int max_bounces;
    long long wave_begin;   // first path index of this wave
    int wave_count;         // paths in this wave
    Queue q[2];
    float2 *hits;
    ShadowQ sq;
    ShadowQ cq;             // carry region of the shadow planes (blocked reference photons)
    int carry_cap;
    float *accum;           // [total slots][4]
    Ctrl *ctrl;
    unsigned long long *counters;  // counting pass only
    int *prefix;                   // adjoint pass only
};

template <bool MULTI>
__device__ __forceinline__ const Item &job_of(const WaveArgs &A, int job) {
    if (MULTI) return A.items[job];
    return A.inl;
}

__device__ __forceinline__ f3 cam_to_world(const dr_camera &c, f3 d) {
    return f3{d.x * c.right[0] + d.y * c.up[0] + d.z * c.forward[0], d.x * c.right[1] + d.y * c.up[1] + d.z * c.forward[1],
              d.x * c.right[2] + d.y * c.up[2] + d.z * c.forward[2]};
}

// Lens sample for one path.  Returns false for pixels that produce no ray.
__device__ inline bool lens_ray(const Item &I, int x, int y, int s, uint32_t key, f3 &o, f3 &d, c3 &filter) {
    const dr_camera &c = I.camera;
    filter = mkc(1, 1, 1);
    if (I.mode == DR_MODE_REFERENCE) {
        int fi = s / I.fsaa_y, fj = s - fi * I.fsaa_y;
        float px = ((float)x - ((float)I.width / 2.0f)) * I.pixel_size;
        float py = (((float)I.height / 2.0f) - (float)y) * I.pixel_size;
        float sx = px + (((float)fi) + 0.5f) * I.pdx;
        float sy = py + (((float)fj) + 0.5f) * I.pdy;
        float ox = I.pdx / 2.0f, oy = I.pdy / 2.0f;
        if (c.lens == DR_LENS_DEFAULT_PERSPECTIVE) {
            o = f3{0, 0, 0};
            d = norm3(f3{sx, sy, I.cam_x});
        } else if (c.lens == DR_LENS_SIMPLE_STOCHASTIC) {
            float jx = (rnd(key, kLensBounce, 0) * (ox - (-ox))) + (-ox);
            float jy = (rnd(key, kLensBounce, 1) * (oy - (-oy))) + (-oy);
            o = f3{0, 0, 0};
            d = f3{sx + jx, sy + jy, I.cam_x};
        } else {
            float jx = (rnd(key, kLensBounce, 0) * (ox - (-ox))) + (-ox);
            float jy = (rnd(key, kLensBounce, 1) * (oy - (-oy))) + (-oy);
            const float RADIAN = 57.29577951308233f;
            float ha = ((sx + jx) * c.angle[0] / RADIAN);
            float va = ((sy + jy) * c.angle[1] / RADIAN);
            f3 td = f3{sinf(ha) * cosf(va), sinf(va), cosf(ha) * cosf(va)};
            f3 target = mul3(td, c.focal_distance);
            float ra = (rnd(key, kLensBounce, 2) * (2.0f * 3.14159265359f - 0.0f)) + 0.0f;
            f3 origin = mul3(mul3(f3{cosf(ra), sinf(ra), 0.0f}, asinf(rnd(key, kLensBounce, 3))), c.softness);
            o = origin;
            d = norm3(sub3(target, origin));
            filter = mkc(c.filter[0], c.filter[1], c.filter[2]);
        }
    } else {
        float jx = rnd(key, kLensBounce, 0), jy = rnd(key, kLensBounce, 1);
        float sx = ((float)x + jx - 0.5f * (float)I.width) / (float)I.height;
        float sy = (0.5f * (float)I.height - ((float)y + jy)) / (float)I.height;
        f3 dl;
        const float PI = 3.14159265358979f;
        if (c.lens == DR_LENS_FISHEYE) {
            float r = sqrtf(sx * sx + sy * sy);
            float theta = r * (c.angle[0] * PI / 180.0f);
            if (theta > PI) return false;
            float phi = atan2f(sy, sx);
            float st = sinf(theta);
            dl = f3{st * cosf(phi), st * sinf(phi), cosf(theta)};
        } else if (c.lens == DR_LENS_SPHERICAL) {
            float h = sx * (c.angle[0] * PI / 180.0f);
            float v = sy * (c.angle[1] * PI / 180.0f);
            dl = f3{sinf(h) * cosf(v), sinf(v), cosf(h) * cosf(v)};
        } else {
            dl = norm3(f3{sx, sy, I.cam_x});
        }
        d = norm3(cam_to_world(c, dl));
        o = f3{c.position[0], c.position[1], c.position[2]};
        return true;
    }
    if (c.origin_rows)
        o = f3{o.x * c.row_x[0] + o.y * c.row_x[1] + o.z * c.row_x[2] + c.position[0],
               o.x * c.row_y[0] + o.y * c.row_y[1] + o.z * c.row_y[2] + c.position[1],
               o.x * c.row_z[0] + o.y * c.row_z[1] + o.z * c.row_z[2] + c.position[2]};
    else
        o = add3(cam_to_world(c, o), f3{c.position[0], c.position[1], c.position[2]});
    d = cam_to_world(c, d);
    return true;
}

// The job owning global path index g (jobs sorted by path_begin).
template <bool MULTI>
__device__ __forceinline__ int job_of_path(const WaveArgs &A, long long g) {
    if (!MULTI) return 0;
    int lo = 0, hi = A.n_items - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (A.items[mid].path_begin <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <bool MULTI>
__global__ void __launch_bounds__(256) k_camera(WaveArgs A) {
    Ctrl *C = A.ctrl;
    for (;;) {
        int base = warp_fetch(&C->fetch_camera);
        if (base >= A.wave_count) break;
        int i = base + (int)lane_id();
        bool valid = i < A.wave_count;
        f3 o = f3{0, 0, 0}, d = f3{0, 0, 1};
        c3 filt = mkc(0, 0, 0);
        int slot = 0, pixel = 0, job = 0;
        uint32_t sample = 0;
        if (valid) {
            long long g = A.wave_begin + i;
            job = job_of_path<MULTI>(A, g);
            const Item &I = job_of<MULTI>(A, job);
            long long lp = g - I.path_begin;
            int s = (int)(lp / I.n_slots);
            int lslot = (int)(lp - (long long)s * I.n_slots);
            slot = I.slot_begin + lslot;
            int blk = I.start_block + lslot / (DR_BLOCK_W * DR_BLOCK_H);
            int pid = lslot % (DR_BLOCK_W * DR_BLOCK_H);
            int bw = (I.width + DR_BLOCK_W - 1) / DR_BLOCK_W;
            int by = blk / bw, bx = blk - by * bw;
            int x = bx * DR_BLOCK_W + (pid % DR_BLOCK_W), y = by * DR_BLOCK_H + pid / DR_BLOCK_W;
            valid = (x < I.width) && (y < I.height);
            if (valid) {
                pixel = y * I.width + x;
                sample = I.sample_base + (uint32_t)s;
                uint32_t key = path_key(I.seed, (uint32_t)pixel, sample);
                valid = lens_ray(I, x, y, s, key, o, d, filt);
            }
        }
        int w = warp_alloc(&C->ray_count[0], valid);
        if (valid) {
            Queue &Q = A.q[0];
            Q.p0[w] = make_float4(o.x, o.y, o.z, __int_as_float(slot));
            Q.p1[w] = make_float4(d.x, d.y, d.z, __uint_as_float(sample));
            Q.p2[w] = make_float4(filt.r, filt.g, filt.b, 0.0f);
            Q.p3[w] = make_int4(-1, 1 | (i << 1), pixel, job);
        }
    }
}

// Traversal steps a lane may take between two cooperative leaf rounds on physical-tree scenes
// (small leaves; the reference's tree keeps 1).  Path trace of the open 1.31M-triangle scene at leaf
// split 4, Mpaths/s: 1: 654, 2: 789, 3: 795, 4: 810, 6: 723, 8: 648; but 4 slowed the closed scenes
// (box rooms: adjoint forward 43.5 -> 51.5 ms, 64-scene batch 405 -> 378 Mpaths/s), so it stays 2.
constexpr int kPhysStepsPerRound = 2;

template <bool MULTI>
struct TraceSource {
    static constexpr float kOccludeBelow = 0.0f;
    const WaveArgs *A;
    Queue Q;
    float2 *hits;
    int *fetch;
    int n, chunk;
    long long rays, nb, nt;
    __device__ __forceinline__ bool next(int &b, int &e) { return fetch_chunk(fetch, n, chunk, b, e); }
    __device__ __forceinline__ bool load(int i, f3 &o, f3 &d, int &ign, int &job) {
        float4 p0 = Q.p0[i], p1 = Q.p1[i];
        int4 p3 = Q.p3[i];
        o = f3of(p0);
        d = f3of(p1);
        ign = p3.x;
        job = p3.w;
        return true;
    }
    __device__ __forceinline__ const Scene &scene(int job) { return job_of<MULTI>(*A, job).S; }
    __device__ __forceinline__ bool clip(int job) {
        const Item &I = job_of<MULTI>(*A, job);
        return I.mode == DR_MODE_REFERENCE && I.clip != 0;
    }
    __device__ __forceinline__ bool store(int i, const Hit &h, int b_, int t_) {
        hits[i] = make_float2(__int_as_float(h.tri), h.t);
        rays++;
        nb += b_;
        nt += t_;
        return false;
    }
};

// Block shape of the traversal kernels (k_trace, k_shadow_phys): 8 warps, 3 blocks per SM caps
// registers at 80 (24 warps per SM); the traversal state needs about that many without spilling.
// Measured on the 1080p path trace (Mpaths/s): 256x3 205.7, 128x6 205.4 (80 registers), 128x7 199.8
// and 64x13 199.8 (72 registers, spills).
constexpr int kTraceThreads = 256;
constexpr int kTraceBlocksPerSM = 3;

// Block shapes a renderer can select (dr_renderer_set_block_shape): 0 = 256 x 3, 1 = 128 x 6 per SM
// (both cap registers at 80); the autotuner times them.
template <bool COUNT, bool MULTI, int TT = kTraceThreads, int TB = kTraceBlocksPerSM>
__global__ void __launch_bounds__(TT, TB) k_trace(WaveArgs A, int b) {
    Ctrl *C = A.ctrl;
    const int n = *((volatile int *)&C->ray_count[b]);
    uint32_t stack[kStack];
    __shared__ WarpLeafSlots slots[TT / 32];
    TraceSource<MULTI> src{&A, A.q[b & 1], A.hits, &C->fetch_trace[b], n, chunk_for(n), 0, 0, 0};
    trace_persistent<COUNT, MULTI>(A.inl.S, src, stack, slots[threadIdx.x >> 5], A.inl.S.front_only ? kPhysStepsPerRound : 1);
    if (COUNT) count_add64(A.counters, src.rays, src.nb, src.nt);
}

// Reference semantics: one layer of DumbRenderer's state machine, with the layer gather folded
// into a forward throughput (getReflectedColor is linear in the photon colour).
template <bool MULTI>
__global__ void __launch_bounds__(kShadeThreads) k_shade_ref(WaveArgs A, int b) {
    Ctrl *C = A.ctrl;
    const Queue Q = A.q[b & 1];
    const Queue N = A.q[(b + 1) & 1];
    const int n = *((volatile int *)&C->ray_count[b]);
    __shared__ ShadeBlockShared bs;
    for (;;) {
        const int base = block_fetch(&C->fetch_shade[b], bs);
        if (base >= n) break;
        int i = base + (int)threadIdx.x;
        bool active = i < n;
        int tri = -1;
        float4 p0, p1, p2;
        int4 p3 = make_int4(0, 0, 0, 0);
        float t = 0.0f;
        if (active) {
            float2 h = A.hits[i];
            tri = __float_as_int(h.x);
            t = h.y;
            p0 = Q.p0[i];
            p1 = Q.p1[i];
            p2 = Q.p2[i];
            p3 = Q.p3[i];
        }
        active = active && tri >= 0;
        const Item &I = job_of<MULTI>(A, p3.w);
        const Scene &S = I.S;
        bool child = false;
        f3 hp = f3{0, 0, 0}, cd = f3{0, 0, 0};
        c3 thr = mkc(0, 0, 0);
        uint32_t key = 0;
        if (active) {
            f3 o = f3of(p0), d = f3of(p1);
            hp = xadd(o, xmul(d, t));
            thr = mkc(p2.x, p2.y, p2.z);
            key = path_key(I.seed, (uint32_t)p3.z, __float_as_uint(p1.w));
            if (b < I.max_bounces) {
                const Material &m = S.mats[__ldg(S.mat_id + tri)];
                TriV v = load_tri(S.tris, tri), nt = load_tri(S.nrms, tri);
                int ctype = 0;
                if (m.type == 0) child = dumb_based_request(S, tri, m, v, nt, hp, d, key, (uint32_t)b, cd, ctype);
                else if (m.type == DR_MAT_FRESNEL) child = false;
                else if (m.type == DR_MAT_DEFAULT) {
                    cd = default_request(v, nt, hp, d);
                    child = true;
                } else {
                    cd = ss_request(m, v, nt, hp, d, key, (uint32_t)b);
                    child = true;
                }
                if (child) {
                    c3 w = ref_reflect(S, tri, hp, neg3(cd), neg3(d), false, ctype);
                    p2 = make_float4(thr.r * w.r, thr.g * w.g, thr.b * w.b, 0.0f);  // throughput of the child layer
                }
            }
        }
        // light photons: one shadow record per photon of each light of the path's scene (a
        // spotlight sends `samples` photons); photons of a light that casts no shadows are added
        // at once (DumbRenderer.cu:300-316: no cast, every photon illuminates)
        const int n_lights = MULTI ? 16 : A.inl.S.n_lights;
        for (int li = 0; li < n_lights; li++) {
            const bool has = active && li < S.n_lights;
            if (MULTI && !__any_sync(0xFFFFFFFFu, has)) break;
            const int cnt = has ? light_photons(S.lights[li]) : 0;
            const int kmax = __reduce_max_sync(0xFFFFFFFFu, cnt);
            for (int k = 0; k < kmax; k++) {
                bool emit = false;
                f3 lo, ld;
                c3 lc, contrib;
                if (k < cnt) {
                    const Light &L = S.lights[li];
                    bool ok = true;
                    if (L.type == DR_LIGHT_SPOTLIGHT) ok = spot_photon(L, hp, key, (uint32_t)b, li, k, lo, ld, lc);
                    else light_photon(L, hp, key, (uint32_t)b, li, lo, ld, lc);
                    if (ok) {
                        c3 r = ref_reflect(S, tri, hp, ld, neg3(f3of(p1)), true, 0);
                        contrib = cmul(thr, r);
                        emit = (contrib.r + contrib.g + contrib.b) != 0.0f && (lc.r + lc.g + lc.b) != 0.0f;
                        if (emit && L.type == DR_LIGHT_SPOTLIGHT && !L.shadows) {
                            accum_add(A.accum, __float_as_int(p0.w), cmul(contrib, lc));
                            emit = false;
                        }
                    }
                }
                int w = warp_alloc(&C->shadow_count[b], emit);
                if (emit) {
                    A.sq.s0[w] = make_float4(lo.x, lo.y, lo.z, p0.w);
                    A.sq.s1[w] = make_float4(ld.x, ld.y, ld.z, __int_as_float(tri));
                    A.sq.s2[w] = make_float4(hp.x, hp.y, hp.z, __int_as_float(-1));
                    A.sq.s3[w] = make_float4(lc.r, lc.g, lc.b, 0.0f);
                    A.sq.s4[w] = make_float4(contrib.r, contrib.g, contrib.b, __int_as_float(p3.w));
                }
            }
        }
        int w = block_alloc_by_octant(&C->ray_count[b + 1], child, cd, bs);
        if (child) {
            N.p0[w] = make_float4(hp.x, hp.y, hp.z, p0.w);
            N.p1[w] = make_float4(cd.x, cd.y, cd.z, p1.w);
            N.p2[w] = p2;
            N.p3[w] = make_int4(tri, p3.y & ~1, p3.z, p3.w);
        }
    }
}

// Reference light visibility (DumbRenderer.cu:361-428): cast from the light sample toward the
// point; it counts if the first hit is the shaded triangle or lies within sqrt(8 eps) of the
// point; otherwise the blocker's reflected colour decides whether the photon continues (from just
// past the blocker, with that colour, the blocker as the ignored object).
//
// The casts run on the persistent traversal engine.  k_shadow_ref casts every photon of a bounce
// once and settles those that arrive or miss; a photon stopped by a blocker becomes a blocked record
// (the hit point in s0, the blocker in s2.w, its cast count negated in s3.w) in the wave's carry
// region.  k_photon_chain, once per wave after the last bounce, takes the blocked photons: the
// blocker's colour decides whether each continues, and a continuing photon starts its next cast at
// once in the same lane (its record rewritten in place, the engine's restart), so a chain of any
// length keeps its lane.  Under 1% of the photons of the path-trace twin are ever blocked, but
// compiled into the cast kernel the blocker shading and the chain restart cost every cast, and a
// chain launch per bounce would end every bounce with its longest chain; so the cast kernel holds
// no shading code and the chains wait for the wave's end.  When the carry region is full a blocked
// photon stays in its bounce's record and joins the bounce's blocked list (in the spent extension
// queue), which a k_photon_chain launch right after the bounce's casts takes (an empty launch
// otherwise).  Chains read nothing that later bounces write, so neither order changes a result.
// At most kPhotonCasts casts per photon (the oracle's bound, never reached by a photon that moves
// along one line through finite geometry); the count travels in s3.w.
constexpr int kPhotonCasts = 64;

__device__ __forceinline__ bool photon_arrives(const Hit &h, int target, f3 hp) {
    const f3 dd = xsub(h.p, hp);
    return h.tri == target || xdot(dd, dd) <= (8.0f * kEps);
}

// The blocker's transparency colour of a photon cast: shading called out of line, so that its
// registers do not weigh on the traversal it is reached from.
__device__ __noinline__ c3 blocker_reflect(const Scene &S, int tri, f3 p, f3 ld) { return ref_reflect(S, tri, p, ld, ld, true, 0); }

// Blocked photon lists live in the bounce's spent extension queue: in reference mode nothing reads
// q[b & 1] between k_shade_ref(b) and k_shade_ref(b + 1), and its p0 plane (4 ints per path) holds
// the bounce's photons (at most 2 per path of the wave's capacity).
__device__ __forceinline__ int *blocked_list(const WaveArgs &A, int b) { return reinterpret_cast<int *>(A.q[b & 1].p0); }

// Photon j, stopped by blocker `tri` at `p` after `casts` casts: the blocker's reflected colour
// decides whether it continues; if so its record becomes the next cast.  False: the photon ends.
template <bool MULTI>
__device__ __forceinline__ bool photon_pass(const WaveArgs &A, const ShadowQ &sq, int j, int tri, f3 p, int casts) {
    const float4 s3 = sq.s3[j];
    const Scene &S = job_of<MULTI>(A, __float_as_int(sq.s4[j].w)).S;
    const f3 ld = f3of(sq.s1[j]);
    const c3 tr = cmul(blocker_reflect(S, tri, p, ld), mkc(s3.x, s3.y, s3.z));
    if (!((tr.r + tr.g + tr.b) > kEps)) return false;
    const f3 lo = add3(p, mul3(norm3(ld), 64.0f * kEps));
    sq.s0[j] = make_float4(lo.x, lo.y, lo.z, sq.s0[j].w);
    const float4 s2 = sq.s2[j];
    sq.s2[j] = make_float4(s2.x, s2.y, s2.z, __int_as_float(tri));
    sq.s3[j] = make_float4(tr.r, tr.g, tr.b, __int_as_float(casts));
    return true;
}

// An arriving photon adds its colour to its pixel's accumulator.
__device__ __forceinline__ void photon_arrive(const WaveArgs &A, const ShadowQ &sq, int j) {
    const float4 s3 = sq.s3[j], s4 = sq.s4[j];
    accum_add(A.accum, __float_as_int(sq.s0[j].w), mkc(s4.x * s3.x, s4.y * s3.y, s4.z * s3.z));
}

// First cast of every photon of a bounce (k_shadow_ref).
template <bool MULTI>
struct RefPhotonSource {
    static constexpr float kOccludeBelow = 0.0f;
    const WaveArgs *A;
    ShadowQ sq;
    int *fetch;
    int *carry_count;
    int *blocked, *blocked_count;
    int n, chunk;
    long long rays, nb, nt;
    __device__ __forceinline__ bool next(int &b, int &e) { return fetch_chunk(fetch, n, chunk, b, e); }
    __device__ __forceinline__ bool load(int i, f3 &o, f3 &d, int &ign, int &job) {
        o = f3of(sq.s0[i]);
        d = f3of(sq.s1[i]);
        ign = __float_as_int(sq.s2[i].w);
        job = __float_as_int(sq.s4[i].w);
        return true;
    }
    __device__ __forceinline__ const Scene &scene(int job) { return job_of<MULTI>(*A, job).S; }
    __device__ __forceinline__ bool clip(int job) { return job_of<MULTI>(*A, job).clip != 0; }
    __device__ __forceinline__ bool store(int i, const Hit &h, int b_, int t_) {
        rays++;
        nb += b_;
        nt += t_;
        if (h.tri < 0) return false;
        const float4 s2 = sq.s2[i];
        if (photon_arrives(h, __float_as_int(sq.s1[i].w), f3of(s2))) {
            photon_arrive(*A, sq, i);
            return false;
        }
        const float4 s3 = sq.s3[i];
        const int casts = __float_as_int(s3.w) + 1;
        if (casts >= kPhotonCasts) return false;
        const float4 b0 = make_float4(h.p.x, h.p.y, h.p.z, sq.s0[i].w);
        const float4 b2 = make_float4(s2.x, s2.y, s2.z, __int_as_float(h.tri));
        const float4 b3 = make_float4(s3.x, s3.y, s3.z, __int_as_float(-casts));
        const int k = atomicAdd(carry_count, 1);
        if (k < A->carry_cap) {
            const ShadowQ &cq = A->cq;
            cq.s0[k] = b0;
            cq.s1[k] = sq.s1[i];
            cq.s2[k] = b2;
            cq.s3[k] = b3;
            cq.s4[k] = sq.s4[i];
        } else {
            sq.s0[i] = b0;
            sq.s2[i] = b2;
            sq.s3[i] = b3;
            blocked[atomicAdd(blocked_count, 1)] = i;
        }
        return false;
    }
};

// Blocked photons and their chains (k_photon_chain): entry i is record blocked[i] of `sq` (a
// bounce's records), or record i when `blocked` is null (the carry region).
template <bool MULTI>
struct RefPhotonChainSource {
    static constexpr float kOccludeBelow = 0.0f;
    const WaveArgs *A;
    ShadowQ sq;
    const int *blocked;
    int *fetch;
    int n, chunk;
    long long rays, nb, nt;
    __device__ __forceinline__ bool next(int &b, int &e) { return fetch_chunk(fetch, n, chunk, b, e); }
    __device__ __forceinline__ bool load(int i, f3 &o, f3 &d, int &ign, int &job) {
        const int j = blocked ? blocked[i] : i;
        const int w = __float_as_int(sq.s3[j].w);
        if (w < 0 && !photon_pass<MULTI>(*A, sq, j, __float_as_int(sq.s2[j].w), f3of(sq.s0[j]), -w)) return false;
        o = f3of(sq.s0[j]);
        d = f3of(sq.s1[j]);
        ign = __float_as_int(sq.s2[j].w);
        job = __float_as_int(sq.s4[j].w);
        return true;
    }
    __device__ __forceinline__ const Scene &scene(int job) { return job_of<MULTI>(*A, job).S; }
    __device__ __forceinline__ bool clip(int job) { return job_of<MULTI>(*A, job).clip != 0; }
    __device__ __forceinline__ bool store(int i, const Hit &h, int b_, int t_) {
        rays++;
        nb += b_;
        nt += t_;
        if (h.tri < 0) return false;
        const int j = blocked ? blocked[i] : i;
        if (photon_arrives(h, __float_as_int(sq.s1[j].w), f3of(sq.s2[j]))) {
            photon_arrive(*A, sq, j);
            return false;
        }
        const int casts = __float_as_int(sq.s3[j].w) + 1;
        if (casts >= kPhotonCasts) return false;
        return photon_pass<MULTI>(*A, sq, j, h.tri, h.p, casts);
    }
};

// Blocks per SM of the photon kernels (kTraceThreads threads each): the first-cast kernel holds no
// shading and takes the traversal's own budget; the chain kernel, with the blocker shading, gets up
// to 128 registers.
constexpr int kShadowRefBlocksPerSM = 3;
constexpr int kPhotonChainBlocksPerSM = 2;

template <bool COUNT, bool MULTI>
__global__ void __launch_bounds__(kTraceThreads, kShadowRefBlocksPerSM) k_shadow_ref(WaveArgs A, int b) {
    Ctrl *C = A.ctrl;
    const int n = *((volatile int *)&C->shadow_count[b]);
    if (n == 0) return;
    uint32_t stack[kStack];
    __shared__ WarpLeafSlots slots[kTraceThreads / 32];
    RefPhotonSource<MULTI> src{&A, A.sq, &C->fetch_shadow[b], &C->carry_count, blocked_list(A, b), &C->blocked_count[b], n,
                               chunk_for(n), 0, 0, 0};
    trace_persistent<COUNT, MULTI>(A.inl.S, src, stack, slots[threadIdx.x >> 5]);
    if (COUNT) count_add64(A.counters + 3, src.rays, src.nb, src.nt);
}

// b >= 0: bounce b's blocked list (photons the full carry region turned away); b < 0: the carry
// region, after the wave's last bounce.
template <bool COUNT, bool MULTI>
__global__ void __launch_bounds__(kTraceThreads, kPhotonChainBlocksPerSM) k_photon_chain(WaveArgs A, int b) {
    Ctrl *C = A.ctrl;
    const bool carry = b < 0;
    const int n = carry ? min(*((volatile int *)&C->carry_count), A.carry_cap) : *((volatile int *)&C->blocked_count[b]);
    if (n == 0) return;
    uint32_t stack[kStack];
    __shared__ WarpLeafSlots slots[kTraceThreads / 32];
    RefPhotonChainSource<MULTI> src{&A, carry ? A.cq : A.sq, carry ? nullptr : blocked_list(A, b),
                                    carry ? &C->fetch_carry : &C->fetch_chain[b], n, chunk_for(n), 0, 0, 0};
    trace_persistent<COUNT, MULTI>(A.inl.S, src, stack, slots[threadIdx.x >> 5]);
    if (COUNT) count_add64(A.counters + 3, src.rays, src.nb, src.nt);
}

// Adjoint helpers: dL/dI of the pixel behind an accumulator slot, divided by spp (the pixel is the
// mean of its samples).
__device__ __forceinline__ c3 pixel_adjoint(const Item &I, int slot) {
    int lslot = slot - I.slot_begin;
    const float4 g = __ldg(reinterpret_cast<const float4 *>(I.dl_dfb) + (size_t)I.start_block * (DR_BLOCK_W * DR_BLOCK_H) + lslot);
    return mkc(g.x * I.inv_spp, g.y * I.inv_spp, g.z * I.inv_spp);
}
// A contribution c (per channel) carrying the albedo factors of path vertices prefix[0..last]:
// d c / d albedo_k = c / albedo_k for each such vertex (every material scales the throughput, and
// the NEE BSDF, linearly by its albedo).
__device__ __forceinline__ void scatter_albedo(const Item &I, const int *pre, int last, c3 delta, c3 c) {
    const float gr = delta.r * c.r, gg = delta.g * c.g, gb = delta.b * c.b;
    if (gr == 0.0f && gg == 0.0f && gb == 0.0f) return;
    for (int j = 0; j <= last; j++) {
        int k = pre[j];
        const float *a = I.S.albedo + 3 * (size_t)k;
        float ar = __ldg(a), ag = __ldg(a + 1), ab = __ldg(a + 2);
        float *g = I.grad_albedo + 3 * (size_t)k;
        if (ar > 1e-8f && gr != 0.0f) atomicAdd(g, gr / ar);
        if (ag > 1e-8f && gg != 0.0f) atomicAdd(g + 1, gg / ag);
        if (ab > 1e-8f && gb != 0.0f) atomicAdd(g + 2, gb / ab);
    }
}

// Physical path step.  ADJ: adjoint pass (no image; gradients of emission hits are scattered here,
// vertex triangles are recorded for the NEE gradients scattered by k_shadow_phys).
template <bool MULTI, bool ADJ>
__global__ void __launch_bounds__(kShadeThreads) k_shade_phys(WaveArgs A, int b) {
    Ctrl *C = A.ctrl;
    const Queue Q = A.q[b & 1];
    const Queue N = A.q[(b + 1) & 1];
    const int n = *((volatile int *)&C->ray_count[b]);
    __shared__ ShadeBlockShared bs, bss;  // fetch + extension rays; shadow rays
    for (;;) {
        const int base = block_fetch(&C->fetch_shade[b], bs);
        if (base >= n) break;
        int i = base + (int)threadIdx.x;
        bool active = i < n;
        int tri = -1;
        float4 p0, p1, p2;
        int4 p3 = make_int4(0, 0, 0, 0);
        float t = 0.0f;
        if (active) {
            float2 h = A.hits[i];
            tri = __float_as_int(h.x);
            t = h.y;
            p0 = Q.p0[i];
            p1 = Q.p1[i];
            p2 = Q.p2[i];
            p3 = Q.p3[i];
        }
        active = active && tri >= 0;
        const Item &I = job_of<MULTI>(A, p3.w);
        const Scene &S = I.S;
        bool emit_shadow = false, child = false;
        f3 hp = f3{0, 0, 0}, sdir = f3{0, 0, 0}, nd = f3{0, 0, 0};
        c3 scontrib = mkc(0, 0, 0), thr = mkc(0, 0, 0);
        int light_tri = -1;
        float new_pdf = 0.0f;
        int new_delta = 0;
        int slot = 0;
        const int path = p3.y >> 1;
        if (active) {
            slot = __float_as_int(p0.w);
            f3 o = f3of(p0), d = f3of(p1);
            hp = xadd(o, xmul(d, t));
            thr = mkc(p2.x, p2.y, p2.z);
            uint32_t key = path_key(I.seed, (uint32_t)p3.z, __float_as_uint(p1.w));
            TriV v = load_tri(S.tris, tri);
            f3 outward = tri_normal(v);
            f3 ng = norm3(outward);
            f3 wo = neg3(d);
            if (dot3(ng, wo) < 0) ng = neg3(ng);
            float4 sh = __ldg(S.shade + tri);
            const float *emp = S.emission + 3 * (size_t)tri;
            c3 em = mkc(__ldg(emp), __ldg(emp + 1), __ldg(emp + 2));
            // emission (one-sided, outward side)
            if (em.r + em.g + em.b > 0.0f) {
                f3 out = norm3(outward);
                float cosl = dot3(out, wo);
                if (cosl > 0) {
                    float w = 1.0f;
                    if (!(p3.y & 1) && S.emissive_total > 0) {
                        float pls = __ldg(S.light_pdf + tri) * (t * t * sqr3(d)) / cosl;
                        w = mis2(p2.w, pls);
                    }
                    c3 c = mkc(thr.r * em.r * w, thr.g * em.g * w, thr.b * em.b * w);
                    if (ADJ) {
                        c3 delta = pixel_adjoint(I, slot);
                        float *g = I.grad_emission + 3 * (size_t)tri;
                        if (delta.r != 0.0f) atomicAdd(g, delta.r * thr.r * w);
                        if (delta.g != 0.0f) atomicAdd(g + 1, delta.g * thr.g * w);
                        if (delta.b != 0.0f) atomicAdd(g + 2, delta.b * thr.b * w);
                        if (b > 0) scatter_albedo(I, A.prefix + (size_t)path * kAdjDepth, b - 1, delta, c);
                    } else {
                        accum_add(A.accum, slot, c);
                    }
                }
            }
            if (ADJ) A.prefix[(size_t)path * kAdjDepth + b] = tri;
            if (b < I.max_bounces) {
                int mt = __float_as_int(sh.y);
                const float *ap = S.albedo + 3 * (size_t)tri;
                c3 alb = mkc(__ldg(ap), __ldg(ap + 1), __ldg(ap + 2));
                float alpha = fmaxf(sh.x, 1e-3f);
                if (mt != DR_MAT_MIRROR && S.n_emissive > 0) {
                    float u = rnd(key, (uint32_t)b, 3) * S.emissive_total;
                    int lo = 0, hi = S.n_emissive - 1;
                    while (lo < hi) {
                        int mid = (lo + hi) >> 1;
                        if (__ldg(S.emissive_cdf + mid) < u) lo = mid + 1;
                        else hi = mid;
                    }
                    int li = __ldg(S.emissive + lo);
                    float u1 = rnd(key, (uint32_t)b, 4), u2 = rnd(key, (uint32_t)b, 5);
                    float su = sqrtf(u1);
                    float ba = 1.0f - su, bb = u2 * su;
                    TriV lt = load_tri(S.tris, li);
                    f3 lp = add3(add3(mul3(lt.a, ba), mul3(lt.b, bb)), mul3(lt.c, 1.0f - ba - bb));
                    f3 ldv = sub3(lp, hp);
                    float dist2 = sqr3(ldv);
                    f3 wi = mul3(ldv, 1.0f / sqrtf(dist2));
                    f3 lout = norm3(tri_normal(lt));
                    float cosl = -dot3(lout, wi);
                    float cosi = dot3(ng, wi);
                    if (cosl > 0 && cosi > 0) {
                        const float *lep = S.emission + 3 * (size_t)li;
                        c3 le = mkc(__ldg(lep), __ldg(lep + 1), __ldg(lep + 2));
                        float pls = __ldg(S.light_pdf + li) * dist2 / cosl;
                        c3 f;
                        float pb;
                        if (mt == DR_MAT_GLOSSY) {
                            f3 h = norm3(add3(wi, wo));
                            float ndh = dot3(ng, h), ndo = dot3(ng, wo);
                            float D = ggx_d(ndh, alpha);
                            float G = ggx_g1(ndo, alpha) * ggx_g1(cosi, alpha);
                            float spec = D * G / (4.0f * ndo * cosi);
                            f = cscale(alb, spec);
                            pb = D * ndh / (4.0f * fabsf(dot3(wo, h)));
                        } else {
                            f = cscale(alb, 1.0f / 3.14159265358979f);
                            pb = cosi / 3.14159265358979f;
                        }
                        float w = mis2(pls, pb);
                        float k = cosi / pls * w;
                        scontrib = mkc(thr.r * f.r * le.r * k, thr.g * f.g * le.g * k, thr.b * f.b * le.b * k);
                        emit_shadow = (scontrib.r + scontrib.g + scontrib.b) > 0.0f;
                        sdir = ldv;
                        light_tri = li;
                    }
                }
                float u1 = rnd(key, (uint32_t)b, 1), u2 = rnd(key, (uint32_t)b, 2);
                f3 T, B;
                onb(ng, T, B);
                child = true;
                if (mt == DR_MAT_MIRROR) {
                    nd = sub3(d, mul3(ng, 2.0f * dot3(d, ng)));
                    thr = cmul(thr, alb);
                    new_delta = 1;
                    new_pdf = 0.0f;
                } else if (mt == DR_MAT_GLOSSY) {
                    float phi = 2.0f * 3.14159265358979f * u1;
                    float ct = sqrtf((1.0f - u2) / (1.0f + (alpha * alpha - 1.0f) * u2));
                    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                    f3 h = add3(add3(mul3(T, st * cosf(phi)), mul3(B, st * sinf(phi))), mul3(ng, ct));
                    nd = sub3(mul3(h, 2.0f * dot3(wo, h)), wo);
                    float cosi = dot3(ng, nd);
                    if (cosi <= 0) child = false;
                    else {
                        float ndo = dot3(ng, wo);
                        float G = ggx_g1(ndo, alpha) * ggx_g1(cosi, alpha);
                        float wgt = G * fabsf(dot3(wo, h)) / (ndo * ct);
                        thr = cscale(cmul(thr, alb), wgt);
                        new_pdf = ggx_d(ct, alpha) * ct / (4.0f * fabsf(dot3(wo, h)));
                        new_delta = 0;
                    }
                } else {
                    float r = sqrtf(u1), phi = 2.0f * 3.14159265358979f * u2;
                    float z = sqrtf(fmaxf(0.0f, 1.0f - u1));
                    nd = add3(add3(mul3(T, r * cosf(phi)), mul3(B, r * sinf(phi))), mul3(ng, z));
                    thr = cmul(thr, alb);
                    new_pdf = z / 3.14159265358979f;
                    new_delta = 0;
                }
                if (child) nd = norm3(nd);
            }
        }
        int ws = block_alloc_by_octant(&C->shadow_count[b], emit_shadow, sdir, bss);
        if (emit_shadow) {
            A.sq.s0[ws] = make_float4(hp.x, hp.y, hp.z, __int_as_float(slot));
            A.sq.s1[ws] = make_float4(sdir.x, sdir.y, sdir.z, __int_as_float(light_tri));
            A.sq.s2[ws] = make_float4(0.f, 0.f, 0.f, __int_as_float(tri));
            if (ADJ) A.sq.s3[ws] = make_float4(__int_as_float(path), __int_as_float(b), 0.0f, 0.0f);
            A.sq.s4[ws] = make_float4(scontrib.r, scontrib.g, scontrib.b, __int_as_float(p3.w));
        }
        int w = block_alloc_by_octant(&C->ray_count[b + 1], child, nd, bs);
        if (child) {
            N.p0[w] = make_float4(hp.x, hp.y, hp.z, p0.w);
            N.p1[w] = make_float4(nd.x, nd.y, nd.z, p1.w);
            N.p2[w] = make_float4(thr.r, thr.g, thr.b, new_pdf);
            N.p3[w] = make_int4(tri, (p3.y & ~1) | new_delta, p3.z, p3.w);
        }
    }
}

template <bool MULTI, bool ADJ>
struct ShadowPhysSource {
    // visible unless something but the light triangle is hit before t = 0.999 (store below)
    static constexpr float kOccludeBelow = 0.999f;
    const WaveArgs *A;
    ShadowQ sq;
    float *accum;
    int *fetch;
    int n, chunk;
    long long rays, nb, nt;
    __device__ __forceinline__ bool next(int &b, int &e) { return fetch_chunk(fetch, n, chunk, b, e); }
    __device__ __forceinline__ bool load(int i, f3 &o, f3 &d, int &ign, int &job) {
        o = f3of(sq.s0[i]);
        d = f3of(sq.s1[i]);
        ign = __float_as_int(sq.s2[i].w);
        job = __float_as_int(sq.s4[i].w);
        return true;
    }
    __device__ __forceinline__ const Scene &scene(int job) { return job_of<MULTI>(*A, job).S; }
    __device__ __forceinline__ bool clip(int) { return false; }
    __device__ __forceinline__ bool store(int i, const Hit &h, int b_, int t_) {
        int light_tri = __float_as_int(sq.s1[i].w);
        bool vis = (h.tri < 0) || (h.tri == light_tri) || !(h.t < 0.999f);
        if (vis) {
            if (ADJ) {
                reinterpret_cast<float *>(sq.s2 + i)[0] = 1.0f;  // visible: k_adj_shadow scatters its gradients
            } else {
                float4 s4 = sq.s4[i];
                accum_add(accum, __float_as_int(sq.s0[i].w), mkc(s4.x, s4.y, s4.z));
            }
        }
        rays++;
        nb += b_;
        nt += t_;
        return false;
    }
};

// Adjoint pass: gradients of the visible NEE contributions of bounce b (k_shadow_phys<ADJ> marks a
// visible record with s2.x = 1; k_shade_phys writes s2 = {0, 0, 0, tri}), scattered here rather
// than in the traversal kernel, whose registers then stay the traversal's.
template <bool MULTI>
__global__ void __launch_bounds__(256) k_adj_shadow(WaveArgs A, int b) {
    const int n = *((volatile int *)&A.ctrl->shadow_count[b]);
    for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < n; i += (int)(gridDim.x * blockDim.x)) {
        if (A.sq.s2[i].x == 0.0f) continue;
        const float4 s4 = A.sq.s4[i];
        const c3 c = mkc(s4.x, s4.y, s4.z);
        const Item &I = job_of<MULTI>(A, __float_as_int(s4.w));
        const float4 s3 = A.sq.s3[i];
        const int path = __float_as_int(s3.x), vtx = __float_as_int(s3.y);
        const int light_tri = __float_as_int(A.sq.s1[i].w);
        const c3 delta = pixel_adjoint(I, __float_as_int(A.sq.s0[i].w));
        const float *lep = I.S.emission + 3 * (size_t)light_tri;
        const float lr = __ldg(lep), lg = __ldg(lep + 1), lb = __ldg(lep + 2);
        float *g = I.grad_emission + 3 * (size_t)light_tri;
        if (lr > 0.0f && delta.r != 0.0f) atomicAdd(g, delta.r * c.r / lr);
        if (lg > 0.0f && delta.g != 0.0f) atomicAdd(g + 1, delta.g * c.g / lg);
        if (lb > 0.0f && delta.b != 0.0f) atomicAdd(g + 2, delta.b * c.b / lb);
        scatter_albedo(I, A.prefix + (size_t)path * kAdjDepth, vtx, delta, c);
    }
}

// Physical visibility: closest hit from the shading point toward the sampled light point
// (direction = light point - shading point, so the light is at t = 1), ignoring the shading
// triangle; visible if nothing but the light triangle is hit before t = 0.999.
template <bool COUNT, bool MULTI, bool ADJ, int TT = kTraceThreads, int TB = kTraceBlocksPerSM>
__global__ void __launch_bounds__(TT, TB) k_shadow_phys(WaveArgs A, int b) {
    Ctrl *C = A.ctrl;
    const int n = *((volatile int *)&C->shadow_count[b]);
    uint32_t stack[kStack];
    __shared__ WarpLeafSlots slots[TT / 32];
    ShadowPhysSource<MULTI, ADJ> src{&A, A.sq, A.accum, &C->fetch_shadow[b], n, chunk_for(n), 0, 0, 0};
    trace_persistent<COUNT, MULTI>(A.inl.S, src, stack, slots[threadIdx.x >> 5], A.inl.S.front_only ? kPhysStepsPerRound : 1);
    if (COUNT) count_add64(A.counters + 3, src.rays, src.nb, src.nt);
}

// Accumulators -> frame buffer: set (blend >= 1) or blend like blendBlockPixelColor.
template <bool MULTI>
__global__ void k_resolve(WaveArgs A, int total_slots) {
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= total_slots) return;
    int job = 0;
    if (MULTI) {
        int lo = 0, hi = A.n_items - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (A.items[mid].slot_begin <= slot) lo = mid;
            else hi = mid - 1;
        }
        job = lo;
    }
    const Item &I = job_of<MULTI>(A, job);
    int lslot = slot - I.slot_begin;
    if (lslot >= I.n_slots) return;
    int blk = I.start_block + lslot / (DR_BLOCK_W * DR_BLOCK_H);
    int pid = lslot % (DR_BLOCK_W * DR_BLOCK_H);
    int bw = (I.width + DR_BLOCK_W - 1) / DR_BLOCK_W;
    int by = blk / bw, bx = blk - by * bw;
    int x = bx * DR_BLOCK_W + (pid % DR_BLOCK_W), y = by * DR_BLOCK_H + pid / DR_BLOCK_W;
    if (x >= I.width || y >= I.height) return;
    float4 a = reinterpret_cast<const float4 *>(A.accum)[slot];
    float4 c = make_float4(a.x * I.inv_spp, a.y * I.inv_spp, a.z * I.inv_spp, 1.0f);
    float4 *fb = reinterpret_cast<float4 *>(I.fb);
    size_t at = (size_t)blk * (DR_BLOCK_W * DR_BLOCK_H) + pid;
    const float blend = I.blend;
    if (blend >= 1.0f) fb[at] = c;
    else {
        float4 old = fb[at];
        fb[at] = make_float4((c.x * blend) + (old.x * (1.0f - blend)), (c.y * blend) + (old.y * (1.0f - blend)),
                             (c.z * blend) + (old.z * (1.0f - blend)), (c.w * blend) + (old.w * (1.0f - blend)));
    }
}

// Arena copy of one scene's nodes: child node index += 8 * group_off, first leaf reference += leaf_off.
__global__ void k_rebase_nodes(float4 *dst, const float4 *src, long long n_nodes, int group_off, int leaf_off) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_nodes; i += (long long)gridDim.x * blockDim.x) {
        float4 lo = src[2 * i], hi = src[2 * i + 1];
        int w = __float_as_int(lo.w);
        w = (w >= 0) ? w + 8 * group_off : ~(~w + leaf_off);
        lo.w = __int_as_float(w);
        dst[2 * i] = lo;
        dst[2 * i + 1] = hi;
    }
}

}  // namespace drd

// ---------------------------------------------------------------------------------------------
// Host launchers
namespace drk {

using namespace drd;

// SM count of the current device, cached per device (renderers on several threads and GPUs launch
// concurrently).
static int sm_count() {
    constexpr int kDevs = 64;
    static std::atomic<int> cache[kDevs] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int v = (dev >= 0 && dev < kDevs) ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (v == 0) {
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        if (v <= 0) v = 148;
        if (dev >= 0 && dev < kDevs) cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

cudaError_t launch_cast(const Scene &S, const float *o, const float *d, const int *ignore, int n, int clip, int *hit_tri,
                        float *hit_t, int *nbox, int *ntri, cudaStream_t stream, long long *launches) {
    if (n <= 0) return cudaSuccess;
    int threads = 128;
    int per_block = (threads / 32) * kChunk;
    int blocks = (n + per_block - 1) / per_block;
    if (nbox || ntri)
        k_cast<true><<<blocks, threads, 0, stream>>>(S, o, d, ignore, n, clip, hit_tri, hit_t, nbox, ntri);
    else
        k_cast<false><<<blocks, threads, 0, stream>>>(S, o, d, ignore, n, clip, hit_tri, hit_t, nullptr, nullptr);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

size_t ctrl_bytes() { return sizeof(Ctrl); }

cudaError_t read_wave_counts(const void *ctrl, int *rays, int *shadows, int n) {
    const Ctrl *C = static_cast<const Ctrl *>(ctrl);
    cudaError_t e = cudaMemcpy(rays, C->ray_count, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(shadows, C->shadow_count, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
    return e;
}

Profiler::~Profiler() {
    reset();
    for (cudaEvent_t e : pool_) cudaEventDestroy(e);
    if (base_) cudaEventDestroy(base_);
}
cudaEvent_t Profiler::take() {
    if (!pool_.empty()) {
        cudaEvent_t e = pool_.back();
        pool_.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
void Profiler::begin(int cls, cudaStream_t s) {
    if (!enabled) return;
    open_[cls] = take();
    cudaEventRecord(open_[cls], s);
}
void Profiler::end(int cls, cudaStream_t s) {
    if (!enabled || !open_[cls]) return;
    cudaEvent_t e = take();
    cudaEventRecord(e, s);
    pending_.push_back({cls, {open_[cls], e}});
    open_[cls] = nullptr;
    launches[cls]++;
}
cudaError_t Profiler::harvest() {
    cudaError_t err = cudaSuccess;
    for (auto &p : pending_) {
        cudaError_t e = cudaEventSynchronize(p.second.second);
        float t = 0.0f, t0 = 0.0f, t1 = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, p.second.first, p.second.second);
        if (e == cudaSuccess && base_) {
            e = cudaEventElapsedTime(&t0, base_, p.second.first);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t1, base_, p.second.second);
        }
        if (e != cudaSuccess) err = e;
        else {
            ms[p.first] += t;
            if (base_) intervals_[p.first].push_back({t0, t1});
        }
        pool_.push_back(p.second.first);
        pool_.push_back(p.second.second);
    }
    pending_.clear();
    return err;
}
void Profiler::reset(bool base) {
    harvest();
    for (int k = 0; k < KC_COUNT; k++) {
        ms[k] = 0.0;
        launches[k] = 0;
        intervals_[k].clear();
    }
    if (base) {
        // every launch recorded from now on completes after the base event
        if (!base_) cudaEventCreate(&base_);
        cudaDeviceSynchronize();
        cudaEventRecord(base_, 0);
        cudaEventSynchronize(base_);
    }
}
void Profiler::busy(double *out) const {
    for (int k = 0; k < KC_COUNT; k++) {
        std::vector<std::pair<float, float>> iv = intervals_[k];
        std::sort(iv.begin(), iv.end());
        double total = 0.0, lo = 0.0, hi = 0.0;
        bool open = false;
        for (const auto &x : iv) {
            if (!open || x.first > hi) {
                if (open) total += hi - lo;
                lo = x.first;
                hi = x.second;
                open = true;
            } else if (x.second > hi) {
                hi = x.second;
            }
        }
        if (open) total += hi - lo;
        out[k] = total;
    }
}

static void fill_args(const WaveDesc &W, WaveArgs &A, unsigned long long *counters) {
    A.inl = W.inl;
    A.items = W.items;
    A.n_items = W.n_items;
    A.max_bounces = W.max_bounces;
    A.wave_begin = W.wave_begin;
    A.wave_count = W.wave_count;
    for (int k = 0; k < 2; k++) {
        A.q[k].p0 = W.q_p0[k];
        A.q[k].p1 = W.q_p1[k];
        A.q[k].p2 = W.q_p2[k];
        A.q[k].p3 = W.q_p3[k];
    }
    A.hits = W.hits;
    A.sq.s0 = W.s[0];
    A.sq.s1 = W.s[1];
    A.sq.s2 = W.s[2];
    A.sq.s3 = W.s[3];
    A.sq.s4 = W.s[4];
    A.carry_cap = carry_capacity(W.shadow_cap);
    A.cq.s0 = W.s[0] + W.shadow_cap;
    A.cq.s1 = W.s[1] + W.shadow_cap;
    A.cq.s2 = W.s[2] + W.shadow_cap;
    A.cq.s3 = W.s[3] + W.shadow_cap;
    A.cq.s4 = W.s[4] + W.shadow_cap;
    A.accum = W.accum;
    A.ctrl = reinterpret_cast<Ctrl *>(W.ctrl);
    A.counters = counters;
    A.prefix = W.prefix;
}

template <bool MULTI, int TT, int TB>
static void launch_wave_t(const WaveDesc &W, const WaveArgs &A, cudaStream_t stream, Profiler &P, bool count, long long &nl) {
    const int grid = sm_count() * 8;
    P.begin(KC_CAMERA, stream);
    k_camera<MULTI><<<grid, 256, 0, stream>>>(A);
    P.end(KC_CAMERA, stream);
    nl++;
    const int tgrid = grid * (256 / TT);   // same threads in flight as the 256-thread kernels
    for (int b = 0; b <= W.max_bounces; b++) {
        P.begin(KC_TRACE, stream);
        if (count) k_trace<true, MULTI, TT, TB><<<tgrid, TT, 0, stream>>>(A, b);
        else k_trace<false, MULTI, TT, TB><<<tgrid, TT, 0, stream>>>(A, b);
        P.end(KC_TRACE, stream);
        P.begin(KC_SHADE, stream);
        if (W.mode == DR_MODE_REFERENCE) k_shade_ref<MULTI><<<grid, kShadeThreads, 0, stream>>>(A, b);
        else if (W.adjoint) k_shade_phys<MULTI, true><<<grid, kShadeThreads, 0, stream>>>(A, b);
        else k_shade_phys<MULTI, false><<<grid, kShadeThreads, 0, stream>>>(A, b);
        P.end(KC_SHADE, stream);
        P.begin(KC_SHADOW, stream);
        if (W.mode == DR_MODE_REFERENCE) {
            const int sgrid = sm_count() * kShadowRefBlocksPerSM;   // one persistent block per slot
            const int cgrid = sm_count() * kPhotonChainBlocksPerSM;
            if (count) {
                k_shadow_ref<true, MULTI><<<sgrid, kTraceThreads, 0, stream>>>(A, b);
                k_photon_chain<true, MULTI><<<cgrid, kTraceThreads, 0, stream>>>(A, b);
            } else {
                k_shadow_ref<false, MULTI><<<sgrid, kTraceThreads, 0, stream>>>(A, b);
                k_photon_chain<false, MULTI><<<cgrid, kTraceThreads, 0, stream>>>(A, b);
            }
            nl++;
        } else if (W.adjoint) {
            k_shadow_phys<false, MULTI, true, TT, TB><<<tgrid, TT, 0, stream>>>(A, b);
            k_adj_shadow<MULTI><<<grid, 256, 0, stream>>>(A, b);
            nl++;
        } else {
            if (count) k_shadow_phys<true, MULTI, false, TT, TB><<<tgrid, TT, 0, stream>>>(A, b);
            else k_shadow_phys<false, MULTI, false, TT, TB><<<tgrid, TT, 0, stream>>>(A, b);
        }
        P.end(KC_SHADOW, stream);
        nl += 3;
    }
    if (W.mode == DR_MODE_REFERENCE) {   // the chains of the wave's blocked photons
        const int cgrid = sm_count() * kPhotonChainBlocksPerSM;
        P.begin(KC_SHADOW, stream);
        if (count) k_photon_chain<true, MULTI><<<cgrid, kTraceThreads, 0, stream>>>(A, -1);
        else k_photon_chain<false, MULTI><<<cgrid, kTraceThreads, 0, stream>>>(A, -1);
        P.end(KC_SHADOW, stream);
        nl++;
    }
}

cudaError_t launch_wave(const WaveDesc &W, cudaStream_t stream, long long *launches, Profiler *prof,
                        unsigned long long *counters) {
    WaveArgs A;
    fill_args(W, A, counters);
    cudaError_t e = cudaMemsetAsync(W.ctrl, 0, sizeof(Ctrl), stream);
    if (e != cudaSuccess) return e;
    long long nl = 0;
    Profiler dummy;
    Profiler &P = prof ? *prof : dummy;
    const bool cnt = counters != nullptr;
    if (W.shape == 1) {
        if (W.items) launch_wave_t<true, 128, 6>(W, A, stream, P, cnt, nl);
        else launch_wave_t<false, 128, 6>(W, A, stream, P, cnt, nl);
    } else {
        if (W.items) launch_wave_t<true, kTraceThreads, kTraceBlocksPerSM>(W, A, stream, P, cnt, nl);
        else launch_wave_t<false, kTraceThreads, kTraceBlocksPerSM>(W, A, stream, P, cnt, nl);
    }
    if (launches) *launches += nl;
    return cudaGetLastError();
}

cudaError_t launch_rebase_nodes(float4 *dst, const float4 *src, long long n_nodes, int group_off, int leaf_off,
                                cudaStream_t stream) {
    if (n_nodes <= 0) return cudaSuccess;
    const int grid = (int)std::min<long long>((n_nodes + 255) / 256, (long long)sm_count() * 8);
    drd::k_rebase_nodes<<<grid, 256, 0, stream>>>(dst, src, n_nodes, group_off, leaf_off);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const WaveDesc &W, int total_slots, cudaStream_t stream, long long *launches, Profiler *prof) {
    WaveArgs A;
    fill_args(W, A, nullptr);
    int threads = 256;
    int blocks = (total_slots + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    if (prof) prof->begin(KC_RESOLVE, stream);
    if (W.items) k_resolve<true><<<blocks, threads, 0, stream>>>(A, total_slots);
    else k_resolve<false><<<blocks, threads, 0, stream>>>(A, total_slots);
    if (prof) prof->end(KC_RESOLVE, stream);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

}  // namespace drk
