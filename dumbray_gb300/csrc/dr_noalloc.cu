// dr_noalloc.cu - dr_render_blocks_noalloc: the block renderer for callers that cannot allocate
// device memory while they render.
//
// Who needs it: a real-time or plugin host whose device memory is owned by someone else's pool or
// fixed budget, or a caller on a latency-critical thread where cudaMalloc / cudaFree would
// synchronise the device.
// dr_render_blocks keeps its wavefront queues in a dr_renderer that cudaMallocs them (and grows
// its accumulator on demand); this entry point instead uses one fixed scratch region that lives
// in the library image as a file-scope __device__ array, so a call allocates nothing.
//
// Limits and rules:
//   * the scratch array is DR_NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that loads the library,
//     held until the process exits;
//   * one call renders at most DR_NOALLOC_MAX_BLOCKS (2048) frame-buffer blocks (262,144 pixels);
//     larger ranges are rejected with DR_E_CAPACITY, so callers split the frame into several calls;
//   * paths run in waves of at most 32,768 (fewer with many lights), so large sample counts take
//     proportionally more launches than dr_render_blocks;
//   * every call on a device shares the same array and it keeps the last call's contents: the
//     accumulator and the queue counters are cleared by each call before use, but two calls whose
//     work overlaps on the GPU (different streams, or different host threads) race on the array and
//     corrupt each other's results - serialise them on one stream;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current and caches it; make that first call before any stream capture begins.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/dr_api.h"
#include "dr_internal.h"
#include "dr_kernels.h"
#include "dr_guard.h"

namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

constexpr int kWavePaths = 32768;
constexpr int kShadowRecords = 2 * kWavePaths;
constexpr size_t kQueuePlane = align_up(sizeof(float4) * (size_t)kWavePaths);
constexpr size_t kHits = align_up(sizeof(float2) * (size_t)kWavePaths);
constexpr size_t kShadowPlane = align_up(sizeof(float4) * drd::shadow_plane_records(kShadowRecords));
constexpr size_t kAccum = align_up(sizeof(float4) * (size_t)DR_NOALLOC_MAX_BLOCKS * DR_BLOCK_W * DR_BLOCK_H);
constexpr size_t kCtrl = 64 * 1024;
constexpr size_t kOffQueues = 0;                       // 2 queues x 4 planes
constexpr size_t kOffHits = kOffQueues + 8 * kQueuePlane;
constexpr size_t kOffShadow = kOffHits + kHits;        // 5 planes
constexpr size_t kOffAccum = kOffShadow + 5 * kShadowPlane;
constexpr size_t kOffCtrl = kOffAccum + kAccum;
constexpr size_t kUsed = kOffCtrl + kCtrl;
static_assert(kUsed <= DR_NOALLOC_SCRATCH_BYTES, "no-alloc scratch layout exceeds the array");

// The scratch region.  Host code must not use this name as an address: it is a host-side stand-in;
// the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[DR_NOALLOC_SCRATCH_BYTES];

std::mutex g_addr_lock;
constexpr int kMaxDevices = 64;
unsigned char *g_addr[kMaxDevices] = {nullptr};

dr_status nfail(dr_status s, const std::string &msg) {
    dr_internal_set_error(msg.c_str());
    return s;
}

// Device address of the scratch array on the current device (set up once per device).
cudaError_t scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> guard(g_addr_lock);
    if (g_addr[dev] == nullptr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" dr_status dr_render_blocks_noalloc(const dr_scene *sc, const dr_camera *cam, float *fb, int32_t start_block,
                                              int32_t end_block, const dr_render_params *p, void *stream_ptr) try {
    drk::WaveDesc W;
    std::memset(&W, 0, sizeof(W));
    drk::Item &I = W.inl;
    dr_status st = dr_internal_make_item(sc, cam, fb, start_block, end_block, p, "dr_render_blocks_noalloc", I);
    if (st != DR_OK) return st;
    if (end_block - start_block > DR_NOALLOC_MAX_BLOCKS)
        return nfail(DR_E_CAPACITY, "dr_render_blocks_noalloc: " + std::to_string(end_block - start_block) +
                                        " blocks requested, at most " + std::to_string(DR_NOALLOC_MAX_BLOCKS) +
                                        " per call (split the range)");
    if (drk::ctrl_bytes() > kCtrl) return nfail(DR_E_CAPACITY, "dr_render_blocks_noalloc: control block too large");
    if (start_block == end_block) return DR_OK;
    const drd::Scene *S = dr_internal_scene_device(sc);
    cudaStream_t stream = (cudaStream_t)stream_ptr;

    unsigned char *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return nfail(DR_E_CUDA, std::string("dr_render_blocks_noalloc: scratch set-up: ") + cudaGetErrorString(e));

    const int spp = I.spp;
    const int n_slots = I.n_slots;
    const int per_path_shadow = (p->mode == DR_MODE_REFERENCE) ? std::max(1, S->shadow_photons) : 1;
    long long wave = std::min<long long>(kWavePaths, (long long)kShadowRecords / per_path_shadow);
    wave = std::max<long long>(32, (wave / 32) * 32);

    float *accum = reinterpret_cast<float *>(base + kOffAccum);
    e = cudaMemsetAsync(accum, 0, sizeof(float4) * (size_t)n_slots, stream);
    if (e != cudaSuccess) return nfail(DR_E_CUDA, std::string("dr_render_blocks_noalloc: clear: ") + cudaGetErrorString(e));

    W.items = nullptr;
    W.n_items = 1;
    W.mode = p->mode;
    W.max_bounces = p->max_bounces;
    W.adjoint = false;
    for (int k = 0; k < 2; k++) {
        W.q_p0[k] = reinterpret_cast<float4 *>(base + kOffQueues + (4 * k + 0) * kQueuePlane);
        W.q_p1[k] = reinterpret_cast<float4 *>(base + kOffQueues + (4 * k + 1) * kQueuePlane);
        W.q_p2[k] = reinterpret_cast<float4 *>(base + kOffQueues + (4 * k + 2) * kQueuePlane);
        W.q_p3[k] = reinterpret_cast<int4 *>(base + kOffQueues + (4 * k + 3) * kQueuePlane);
    }
    W.hits = reinterpret_cast<float2 *>(base + kOffHits);
    for (int j = 0; j < 5; j++) W.s[j] = reinterpret_cast<float4 *>(base + kOffShadow + j * kShadowPlane);
    W.shadow_cap = kShadowRecords;
    W.accum = accum;
    W.ctrl = base + kOffCtrl;
    W.prefix = nullptr;
    long long launches = 0;
    const long long total = (long long)n_slots * spp;
    for (long long b = 0; b < total; b += wave) {
        W.wave_begin = b;
        W.wave_count = (int)std::min<long long>(wave, total - b);
        e = drk::launch_wave(W, stream, &launches, nullptr, nullptr);
        if (e != cudaSuccess) return nfail(DR_E_CUDA, std::string("dr_render_blocks_noalloc: wave: ") + cudaGetErrorString(e));
    }
    e = drk::launch_resolve(W, n_slots, stream, &launches, nullptr);
    if (e != cudaSuccess) return nfail(DR_E_CUDA, std::string("dr_render_blocks_noalloc: resolve: ") + cudaGetErrorString(e));
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_render_blocks_noalloc");
}
