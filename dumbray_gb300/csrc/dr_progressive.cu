// dr_progressive.cu - progressive render process: a host thread that renders iteration after
// iteration of one view through dr_render_blocks and publishes every finished image.
//
// It plays the part of BufferedRenderProcess (DataStructures/Renderers/BufferedRenderProcess/
// BufferedRenderProcess.cu:117-229) minus the window: a worker thread loops
//   settings snapshot -> (reset on a settings change) -> render one iteration -> publish -> callbacks
// until stopped, rendering nothing once the target iteration count is reached.  Single-buffered,
// iterations accumulate with the progressive blend 1/i (DumbRenderer.cu:64,102).  Double-buffered,
// like the reference (which swaps buffers and resets the iteration count after each iteration),
// every frame is one fresh iteration: the view is re-rendered continuously for a live preview, each
// frame with its own random numbers (seed + frame index); the published image is always the last
// complete frame while the next one renders in the other device buffer.
//
// The published image is a host row-major float4 copy taken after the iteration completed, so
// readers never see a half-rendered buffer.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/dr_api.h"
#include "dr_guard.h"

void dr_internal_set_error(const char *msg);

struct dr_progressive {
    const dr_scene *scene = nullptr;
    int device = 0;
    bool double_buffered = false;

    std::mutex m;
    std::condition_variable cv;
    std::thread worker;
    bool running = false, stop = false, dirty = true;
    // settings (guarded by m)
    dr_camera camera{};
    dr_render_params params{};
    int target = -1;                 // iterations (single) or frames (double) to render; < 0 = unlimited
    dr_progress_callback on_iteration = nullptr, on_complete = nullptr, on_error = nullptr;
    void *cb_arg = nullptr;
    // progress (guarded by m)
    int done = 0;                    // completed iterations (single) or frames (double) since the last reset
    long long frames = 0;            // frames rendered since creation (double-buffered seeds)
    std::vector<float> front;        // last complete image, row-major float4
    int front_w = 0, front_h = 0, front_iteration = 0;
    std::string error;
    double render_seconds = 0.0;

    // worker-owned device state
    dr_renderer *renderer = nullptr;
    cudaStream_t stream = nullptr;
    float *fb[2] = {nullptr, nullptr};
    float *staging = nullptr;        // pinned host copy of the frame buffer
    size_t fb_floats = 0;
    int back = 0;

    void release_device() {
        for (auto &p : fb) { cudaFree(p); p = nullptr; }
        cudaFreeHost(staging);
        staging = nullptr;
        fb_floats = 0;
    }
    ~dr_progressive() {
        release_device();
        if (renderer) dr_renderer_destroy(renderer);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

dr_status fail(dr_status s, const std::string &msg) {
    dr_internal_set_error(msg.c_str());
    return s;
}

// One iteration (or frame) with the settings `cam`, `p`; fills the host image `img`.
bool render_once(dr_progressive *P, const dr_camera &cam, dr_render_params p, int iteration, long long frame,
                 std::vector<float> &img, std::string &err) {
    const int bw = (p.width + DR_BLOCK_W - 1) / DR_BLOCK_W, bh = (p.height + DR_BLOCK_H - 1) / DR_BLOCK_H;
    const int blocks = bw * bh;
    const size_t floats = (size_t)blocks * DR_BLOCK_W * DR_BLOCK_H * 4;
    if (floats != P->fb_floats) {
        P->release_device();
        for (int k = 0; k < (P->double_buffered ? 2 : 1); k++) {
            if (cudaMalloc((void **)&P->fb[k], floats * sizeof(float)) != cudaSuccess ||
                cudaMemset(P->fb[k], 0, floats * sizeof(float)) != cudaSuccess) {
                err = "frame buffer allocation failed";
                P->release_device();
                return false;
            }
        }
        if (cudaMallocHost((void **)&P->staging, floats * sizeof(float)) != cudaSuccess) {
            err = "staging allocation failed";
            P->release_device();
            return false;
        }
        P->fb_floats = floats;
    }
    float *dst = P->fb[P->double_buffered ? P->back : 0];
    if (P->double_buffered) {
        p.iteration = 1;
        p.seed = p.seed + (uint32_t)frame * 0x9E3779B9u;
    } else {
        p.iteration = iteration;
    }
    if (dr_render_blocks(P->renderer, P->scene, &cam, dst, 0, blocks, &p, P->stream) != DR_OK) {
        err = dr_last_error();
        return false;
    }
    cudaError_t e = cudaMemcpyAsync(P->staging, dst, floats * sizeof(float), cudaMemcpyDeviceToHost, P->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    if (e != cudaSuccess) {
        err = cudaGetErrorString(e);
        (void)cudaGetLastError();
        return false;
    }
    img.resize(4 * (size_t)p.width * p.height);
    dr_image_from_blocks(P->staging, p.width, p.height, img.data());
    if (P->double_buffered) P->back ^= 1;
    return true;
}

// Records an exception that escaped one iteration of the worker (host allocation failure while
// staging or publishing an image, for instance) as the render error and fires the error callback;
// the worker then carries on, as it does after a failed render.
void report_worker_exception(dr_progressive *P, const char *what) noexcept {
    dr_progress_callback cb = nullptr;
    void *arg = nullptr;
    {
        std::lock_guard<std::mutex> lk(P->m);
        try {
            P->error = std::string("progressive worker: ") + what;
        } catch (...) {
            P->error.clear();
        }
        cb = P->on_error;
        arg = P->cb_arg;
    }
    P->cv.notify_all();
    if (cb) cb(arg);
    std::this_thread::sleep_for(std::chrono::milliseconds(8));
}

// One iteration of the worker: waits for work, renders, publishes.  false: the worker must stop.
bool worker_iteration(dr_progressive *P, std::vector<float> &img) {
    {
        dr_camera cam;
        dr_render_params p;
        int next;
        long long frame;
        {
            std::unique_lock<std::mutex> lk(P->m);
            for (;;) {
                if (P->stop) return false;
                if (P->dirty) {
                    P->done = 0;
                    P->dirty = false;
                }
                if (P->target < 0 || P->done < P->target) break;
                P->cv.wait_for(lk, std::chrono::milliseconds(8));   // target reached: idle until a change
            }
            cam = P->camera;
            p = P->params;
            next = P->done + 1;
            frame = P->frames;
        }
        std::string err;
        auto t0 = std::chrono::steady_clock::now();
        const bool ok = render_once(P, cam, p, next, frame, img, err);
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        dr_progress_callback cb_it = nullptr, cb_done = nullptr, cb_err = nullptr;
        void *arg = nullptr;
        {
            std::lock_guard<std::mutex> lk(P->m);
            arg = P->cb_arg;
            if (!ok) {
                P->error = err;
                cb_err = P->on_error;
            } else if (!P->dirty) {   // a settings change during the render discards its image
                P->front.swap(img);
                P->front_w = p.width;
                P->front_h = p.height;
                P->front_iteration = P->double_buffered ? 1 : next;
                P->done = next;
                P->frames++;
                P->render_seconds += dt;
                cb_it = P->on_iteration;
                if (P->target >= 0 && P->done >= P->target) cb_done = P->on_complete;
            }
        }
        P->cv.notify_all();
        if (cb_err) cb_err(arg);
        if (cb_it) cb_it(arg);
        if (cb_done) cb_done(arg);
        if (!ok) std::this_thread::sleep_for(std::chrono::milliseconds(8));
    }
    return true;
}

void worker_loop(dr_progressive *P) {
    cudaSetDevice(P->device);
    std::vector<float> img;
    for (;;) {
        try {
            if (!worker_iteration(P, img)) return;
        } catch (const std::exception &ex) {
            report_worker_exception(P, ex.what());
        } catch (...) {
            report_worker_exception(P, "unknown exception");
        }
    }
}

}  // namespace

extern "C" {

dr_status dr_progressive_create(const dr_scene *scene, const dr_camera *camera, const dr_render_params *params,
                                int32_t double_buffered, dr_progressive **out) try {
    if (!out) return fail(DR_E_ARG, "dr_progressive_create: out is NULL");
    *out = nullptr;
    if (!scene || !camera || !params) return fail(DR_E_ARG, "dr_progressive_create: NULL argument");
    if (params->width <= 0 || params->height <= 0) return fail(DR_E_ARG, "dr_progressive_create: bad resolution");
    dr_progressive *P = new (std::nothrow) dr_progressive();
    if (!P) return fail(DR_E_NOMEM, "dr_progressive_create: out of host memory");
    P->scene = scene;
    P->camera = *camera;
    P->params = *params;
    P->double_buffered = double_buffered != 0;
    cudaGetDevice(&P->device);
    dr_status st = dr_renderer_create(0, &P->renderer);
    if (st != DR_OK) {
        delete P;
        return st;
    }
    if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete P;
        return fail(DR_E_CUDA, "dr_progressive_create: stream");
    }
    *out = P;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_create");
}

dr_status dr_progressive_set_target(dr_progressive *P, int32_t iterations) try {
    if (!P) return fail(DR_E_ARG, "dr_progressive_set_target: NULL");
    {
        std::lock_guard<std::mutex> lk(P->m);
        P->target = iterations;
    }
    P->cv.notify_all();
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_set_target");
}

dr_status dr_progressive_set_view(dr_progressive *P, const dr_camera *camera, const dr_render_params *params) try {
    if (!P) return fail(DR_E_ARG, "dr_progressive_set_view: NULL");
    if (params && (params->width <= 0 || params->height <= 0)) return fail(DR_E_ARG, "dr_progressive_set_view: bad resolution");
    {
        std::lock_guard<std::mutex> lk(P->m);
        if (camera) P->camera = *camera;
        if (params) P->params = *params;
        P->dirty = true;   // restart the accumulation, like the reference on a resolution change
    }
    P->cv.notify_all();
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_set_view");
}

dr_status dr_progressive_set_callbacks(dr_progressive *P, dr_progress_callback on_iteration,
                                       dr_progress_callback on_complete, dr_progress_callback on_error, void *arg) try {
    if (!P) return fail(DR_E_ARG, "dr_progressive_set_callbacks: NULL");
    std::lock_guard<std::mutex> lk(P->m);
    P->on_iteration = on_iteration;
    P->on_complete = on_complete;
    P->on_error = on_error;
    P->cb_arg = arg;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_set_callbacks");
}

dr_status dr_progressive_start(dr_progressive *P) try {
    if (!P) return fail(DR_E_ARG, "dr_progressive_start: NULL");
    std::lock_guard<std::mutex> lk(P->m);
    if (P->running) return DR_OK;
    P->stop = false;
    P->running = true;
    P->worker = std::thread(worker_loop, P);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_start");
}

dr_status dr_progressive_stop(dr_progressive *P) try {
    if (!P) return fail(DR_E_ARG, "dr_progressive_stop: NULL");
    {
        std::lock_guard<std::mutex> lk(P->m);
        if (!P->running) return DR_OK;
        P->stop = true;
    }
    P->cv.notify_all();
    P->worker.join();   // the iteration in flight finishes first
    std::lock_guard<std::mutex> lk(P->m);
    P->running = false;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_stop");
}

dr_status dr_progressive_wait(dr_progressive *P, int32_t count, int32_t timeout_ms) try {
    if (!P) return fail(DR_E_ARG, "dr_progressive_wait: NULL");
    std::unique_lock<std::mutex> lk(P->m);
    const bool ok = P->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                   [&] { return !P->dirty && P->done >= count; });
    if (!ok) return fail(DR_E_TIMEOUT, "dr_progressive_wait: timed out" + (P->error.empty() ? std::string() : " (" + P->error + ")"));
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_wait");
}

int32_t dr_progressive_completed(dr_progressive *P) {
    if (!P) return 0;
    std::lock_guard<std::mutex> lk(P->m);
    return P->done;
}

dr_status dr_progressive_read(dr_progressive *P, float *rgba, int32_t width, int32_t height, int32_t *iteration) try {
    if (!P || !rgba) return fail(DR_E_ARG, "dr_progressive_read: NULL argument");
    std::lock_guard<std::mutex> lk(P->m);
    if (P->front.empty()) return fail(DR_E_STATE, "dr_progressive_read: no image completed yet");
    if (width != P->front_w || height != P->front_h)
        return fail(DR_E_CAPACITY, "dr_progressive_read: the image is " + std::to_string(P->front_w) + "x" + std::to_string(P->front_h));
    std::memcpy(rgba, P->front.data(), P->front.size() * sizeof(float));
    if (iteration) *iteration = P->front_iteration;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_progressive_read");
}

dr_status dr_progressive_save_png(dr_progressive *P, const char *path) try {
    if (!P || !path) return fail(DR_E_ARG, "dr_progressive_save_png: NULL argument");
    std::vector<float> img;
    int w, h;
    {
        std::lock_guard<std::mutex> lk(P->m);
        if (P->front.empty()) return fail(DR_E_STATE, "dr_progressive_save_png: no image completed yet");
        img = P->front;
        w = P->front_w;
        h = P->front_h;
    }
    return dr_image_write_png(img.data(), w, h, path);
} catch (...) {
    return dr_internal_exception("dr_progressive_save_png");
}

double dr_progressive_render_seconds(dr_progressive *P) {
    if (!P) return 0.0;
    std::lock_guard<std::mutex> lk(P->m);
    return P->render_seconds;
}

void dr_progressive_destroy(dr_progressive *P) {
    if (!P) return;
    dr_progressive_stop(P);
    delete P;
}

}  // extern "C"
