// dr_kernels.h - host-visible launch interface of the device kernels (no torch types).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <utility>
#include <vector>
#include "../../include/dr_api.h"
#include "dr_device.cuh"

namespace drd {
constexpr int kMaxBounceSlots = 68;  // bounce limit 64 (DUMB_RENDERER_BOUNCE_LIMIT) + camera + spare
constexpr int kAdjDepth = 66;        // prefix slots per path in the adjoint pass (bounces 0..64)

// Reference photons stopped by a blocker wait for their transparency chains in a carry region of
// the shadow planes, behind the `shadow_cap` photon records of a bounce, until the end of the wave.
constexpr int carry_capacity(int shadow_cap) { return std::max(1024, (shadow_cap / 16 + 31) / 32 * 32); }
constexpr size_t shadow_plane_records(int shadow_cap) { return (size_t)shadow_cap + (size_t)carry_capacity(shadow_cap); }
}

namespace drk {

// One render job of a wave: a scene, a camera, a block range of a frame buffer and the render
// parameters.  A plain dr_render_blocks call is a single job passed inline in the kernel
// arguments; a batch keeps a table of jobs in device memory and every path record carries the
// index of its job, so the paths of many scenes share the same waves.
struct Item {
    drd::Scene S;
    dr_camera camera;
    float cam_x;                 // 0.5 / tan(fov / 2) for the pinhole lenses
    int mode, width, height, fsaa_x, fsaa_y, spp, max_bounces, clip;
    float pixel_size, pdx, pdy;
    uint32_t seed, sample_base;
    int start_block, n_slots;
    int slot_begin;              // first pixel slot of this job in the shared accumulator
    long long path_begin;        // first path index of this job in the wave path space
    float *fb;                   // block-major float4 frame buffer
    float inv_spp, blend;
    const float *dl_dfb;         // adjoint: dL/dI, block-major float4 (null outside the adjoint pass)
    float *grad_albedo;          // adjoint: dL/d albedo, float[n][3]
    float *grad_emission;        // adjoint: dL/d emission, float[n][3]
};

// One wave: paths [wave_begin, wave_begin + wave_count) of the path space of all jobs.
struct WaveDesc {
    Item inl;                    // the job when items == nullptr
    const Item *items;           // device job table (batches) or nullptr
    int n_items;
    int mode, max_bounces;
    long long wave_begin;
    int wave_count;
    float4 *q_p0[2], *q_p1[2], *q_p2[2];
    int4 *q_p3[2];
    float2 *hits;
    float4 *s[5];                // shadow planes of drd::shadow_plane_records(shadow_cap) records
    int shadow_cap;
    float *accum;
    void *ctrl;
    int *prefix;                 // adjoint: [wave capacity][kAdjDepth] triangle of each path vertex
    bool adjoint;
    int shape;                   // traversal block shape: 0 = 256 threads x 3 blocks per SM, 1 = 128 x 6
};

// Kernel classes for per-class timing.
enum KernelClass { KC_CAMERA = 0, KC_TRACE = 1, KC_SHADE = 2, KC_SHADOW = 3, KC_RESOLVE = 4, KC_COUNT = 5 };

// CUDA-event timing of kernel launches on their own stream, accumulated per kernel class: the sum
// of launch durations (ms) and, for launches that overlap on several streams, the busy time (the
// length of the union of a class's launch intervals, measured from a base event that precedes all
// of them).
class Profiler {
  public:
    bool enabled = false;
    ~Profiler();
    void begin(int cls, cudaStream_t s);
    void end(int cls, cudaStream_t s);
    // Waits for the recorded events, adds their elapsed times to ms[], keeps their intervals and
    // recycles them.
    cudaError_t harvest();
    // Clears the totals; with `base`, waits for the device and records the base event.
    void reset(bool base = false);
    // Union length of each class's harvested launch intervals.
    void busy(double *out) const;
    double ms[KC_COUNT] = {0, 0, 0, 0, 0};
    long long launches[KC_COUNT] = {0, 0, 0, 0, 0};

  private:
    cudaEvent_t take();
    std::vector<cudaEvent_t> pool_;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending_;
    std::vector<std::pair<float, float>> intervals_[KC_COUNT];
    cudaEvent_t open_[KC_COUNT] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t base_ = nullptr;
};

size_t ctrl_bytes();
// Per-bounce queue counts of the wave last run on control block `ctrl`: rays[b] = extension rays
// traced at bounce b, shadows[b] = shadow / photon records queued at bounce b (b < n <= kMaxBounceSlots).
cudaError_t read_wave_counts(const void *ctrl, int *rays, int *shadows, int n);

cudaError_t launch_cast(const drd::Scene &S, const float *o, const float *d, const int *ignore, int n, int clip, int *hit_tri,
                        float *hit_t, int *nbox, int *ntri, cudaStream_t stream, long long *launches);
// counters (nullable): 6 x u64 = {trace rays, trace box tests, trace tri tests, shadow casts, shadow box tests, shadow tri tests}
cudaError_t launch_wave(const WaveDesc &W, cudaStream_t stream, long long *launches, Profiler *prof,
                        unsigned long long *counters);
// Copies `n_nodes` octree nodes (float4 pairs) into a batch arena at node group `group_off` (node
// index 8 * group_off), adding the offsets to child node and first-leaf-reference indices.
cudaError_t launch_rebase_nodes(float4 *dst, const float4 *src, long long n_nodes, int group_off, int leaf_off,
                                cudaStream_t stream);
// Frame-buffer resolve of all jobs: `total_slots` pixel slots of the shared accumulator.
cudaError_t launch_resolve(const WaveDesc &W, int total_slots, cudaStream_t stream, long long *launches, Profiler *prof);

}  // namespace drk
