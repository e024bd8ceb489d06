// dr_api.cu - C ABI of the GB300 DumbRay hot path (host side; see include/dr_api.h).
//
// Scene objects are immutable after creation and hold the uploaded octree, triangles and
// materials.  Renderer objects own the wavefront scratch (queues, accumulators) for one caller
// thread / stream at a time.  Every entry point validates its arguments, returns a dr_status and
// records a message for dr_last_error(); none falls back to the CPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <atomic>
#include <vector>
#include <new>
#include <exception>

#include "../../include/dr_api.h"
#include "dr_kernels.h"
#include "octree_build.h"
#include "dr_internal.h"
#include "dr_guard.h"

namespace {

thread_local std::string g_err;

dr_status fail(dr_status s, const std::string &msg) {
    g_err = msg;
    return s;
}
dr_status cuda_fail(cudaError_t e, const char *where) {
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    // Reset the runtime's last-error slot: a non-sticky error reported through the status code must
    // not surface again in the caller's next cudaGetLastError() check.
    (void)cudaGetLastError();
    return DR_E_CUDA;
}

template <class T>
cudaError_t upload(T **dst, const T *src, size_t count) {
    *dst = nullptr;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void **)dst, sizeof(T) * count);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
}

// normalised Triangle::normal() = (c - a) x (b - a) (flat shading default)
void flat_normal(const float *p, float out[3]) {
    float ax = p[0], ay = p[1], az = p[2];
    float cax = p[6] - ax, cay = p[7] - ay, caz = p[8] - az;
    float bax = p[3] - ax, bay = p[4] - ay, baz = p[5] - az;
    float x = cay * baz - bay * caz;
    float y = bax * caz - cax * baz;
    float z = cax * bay - bax * cay;
    float im = 1.0f / std::sqrt(x * x + y * y + z * z);
    out[0] = x * im;
    out[1] = y * im;
    out[2] = z * im;
}

}  // namespace

struct dr_scene {
    drd::Scene dev{};
    std::vector<void *> allocs;
    drb::FlatOctree tree;
    int64_t n = 0;
    std::vector<float> xyz;              // host copy of the triangles
    std::vector<int32_t> mat_id;
    std::vector<dr_material> mats;
    std::vector<float> albedo, emission, roughness;
    float4 *shade = nullptr;
    int *emissive = nullptr;
    float *emissive_cdf = nullptr;
    float *albedo_dev = nullptr;         // per-triangle albedo / emission read by the kernels
    float *emission_dev = nullptr;
    float *light_pdf_dev = nullptr;
    int64_t node_f4 = 0, leaf_f4 = 0;    // float4 counts of the device node and leaf-triangle arrays
    int32_t max_texture = 0;             // largest 1-based texture index the materials use
    int32_t n_textures = 0;
    float4 *texels_dev = nullptr;
    int4 *tex_info_dev = nullptr;
    float2 *uv_dev = nullptr;

    ~dr_scene() {
        for (void *p : allocs) cudaFree(p);
        cudaFree(texels_dev);
        cudaFree(tex_info_dev);
        cudaFree(uv_dev);
        cudaFree(shade);
        cudaFree(emissive);
        cudaFree(emissive_cdf);
        cudaFree(albedo_dev);
        cudaFree(emission_dev);
        cudaFree(light_pdf_dev);
    }
};

struct dr_octree {
    drb::FlatOctree tree;
};

// The scratch of one wave pipeline: double-buffered ray queues, hits, shadow queue, control block.
struct WaveScratch {
    float4 *q[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    int4 *q3[2] = {nullptr, nullptr};
    float2 *hits = nullptr;
    float4 *s[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    void *ctrl = nullptr;
    int *prefix = nullptr;          // adjoint: per-path vertex triangles (allocated by the first adjoint)
    int prefix_paths = 0;
    cudaStream_t stream = nullptr;  // extra lanes only
    cudaEvent_t done = nullptr;     // extra lanes only

    cudaError_t alloc(size_t wave, size_t shadow) {
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 2 && e == cudaSuccess; k++) {
            for (int j = 0; j < 3 && e == cudaSuccess; j++) e = cudaMalloc((void **)&q[k][j], sizeof(float4) * wave);
            if (e == cudaSuccess) e = cudaMalloc((void **)&q3[k], sizeof(int4) * wave);
        }
        if (e == cudaSuccess) e = cudaMalloc((void **)&hits, sizeof(float2) * wave);
        for (int j = 0; j < 5 && e == cudaSuccess; j++)
            e = cudaMalloc((void **)&s[j], sizeof(float4) * drd::shadow_plane_records((int)shadow));
        if (e == cudaSuccess) e = cudaMalloc(&ctrl, drk::ctrl_bytes());
        return e;
    }
    void release() {
        for (int k = 0; k < 2; k++) {
            for (int j = 0; j < 3; j++) cudaFree(q[k][j]);
            cudaFree(q3[k]);
        }
        cudaFree(hits);
        for (auto *p : s) cudaFree(p);
        cudaFree(ctrl);
        cudaFree(prefix);
        if (done) cudaEventDestroy(done);
        if (stream) cudaStreamDestroy(stream);
        *this = WaveScratch();
    }
};

struct dr_renderer {
    int capacity = 0;
    float4 *q[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    int4 *q3[2] = {nullptr, nullptr};
    float2 *hits = nullptr;
    float4 *s[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int shadow_capacity = 0;
    float *accum = nullptr;
    size_t accum_slots = 0;
    void *ctrl = nullptr;
    long long launches = 0;
    drk::Profiler prof;
    unsigned long long *counters = nullptr;
    bool counting = false;
    int *prefix = nullptr;          // adjoint: per-path vertex triangles
    int prefix_paths = 0;
    // Concurrent wave pipelines of dr_render_blocks: the renderer's own scratch on the caller's
    // stream plus lanes - 1 extra scratch sets, each on its own stream, taking alternate waves of
    // one render and adding into the same accumulator (one kernel's tail overlaps another
    // pipeline's work).  Extra lanes are allocated on first use.
    int lanes = 1;
    int shape = 0;                  // traversal block shape (dr_renderer_set_block_shape)
    std::vector<WaveScratch> extra;
    cudaEvent_t fork = nullptr;
    // Identifies the current set of scratch buffers: a new value at creation and whenever a buffer a
    // captured batch graph points into is reallocated (process-unique, so a renderer created at
    // the address of a destroyed one never matches a graph captured for the old one).
    unsigned long long scratch_id = next_scratch_id();

    static unsigned long long next_scratch_id() {
        static std::atomic<unsigned long long> counter{0};
        return ++counter;
    }

    ~dr_renderer() {
        cudaFree(counters);
        cudaFree(prefix);
        for (int k = 0; k < 2; k++) {
            for (int j = 0; j < 3; j++) cudaFree(q[k][j]);
            cudaFree(q3[k]);
        }
        cudaFree(hits);
        for (auto *p : s) cudaFree(p);
        cudaFree(accum);
        cudaFree(ctrl);
        for (auto &l : extra) l.release();
        if (fork) cudaEventDestroy(fork);
    }
};

namespace {

// Per-triangle shading records and the emissive-triangle sampling table (physical mode): triangles
// are picked by emitted power (sum of rgb radiance x area), a point uniformly by area, so the area
// pdf of a point of emitter i is (r+g+b)_i / total power.
dr_status upload_shading(dr_scene *sc) {
    const int64_t n = sc->n;
    std::vector<float4> shade(n);
    std::vector<float> light_pdf(n, 0.0f);
    std::vector<int> em;
    std::vector<float> cdf;
    double total = 0.0;
    for (int64_t i = 0; i < n; i++) {
        int type = sc->mats.empty() ? DR_MAT_LAMBERT : sc->mats[sc->mat_id[i]].type;
        float tbits;
        std::memcpy(&tbits, &type, 4);
        shade[i] = make_float4(sc->roughness[i], tbits, 0.0f, 0.0f);
        float esum = sc->emission[3 * i] + sc->emission[3 * i + 1] + sc->emission[3 * i + 2];
        if (esum > 0.0f) {
            const float *p = &sc->xyz[9 * i];
            double ux = p[3] - p[0], uy = p[4] - p[1], uz = p[5] - p[2];
            double vx = p[6] - p[0], vy = p[7] - p[1], vz = p[8] - p[2];
            double cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
            double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
            total += (double)esum * area;
            em.push_back((int)i);
            cdf.push_back((float)total);
        }
    }
    for (size_t k = 0; k < em.size(); k++) {
        int i = em[k];
        float esum = sc->emission[3 * i] + sc->emission[3 * i + 1] + sc->emission[3 * i + 2];
        light_pdf[i] = (float)((double)esum / total);
    }
    cudaFree(sc->shade);
    cudaFree(sc->emissive);
    cudaFree(sc->emissive_cdf);
    cudaFree(sc->albedo_dev);
    cudaFree(sc->emission_dev);
    cudaFree(sc->light_pdf_dev);
    sc->shade = nullptr;
    sc->emissive = nullptr;
    sc->emissive_cdf = nullptr;
    sc->albedo_dev = nullptr;
    sc->emission_dev = nullptr;
    sc->light_pdf_dev = nullptr;
    cudaError_t e = upload(&sc->shade, shade.data(), shade.size());
    if (e == cudaSuccess) e = upload(&sc->emissive, em.data(), em.size());
    if (e == cudaSuccess) e = upload(&sc->emissive_cdf, cdf.data(), cdf.size());
    if (e == cudaSuccess) e = upload(&sc->albedo_dev, sc->albedo.data(), sc->albedo.size());
    if (e == cudaSuccess) e = upload(&sc->emission_dev, sc->emission.data(), sc->emission.size());
    if (e == cudaSuccess) e = upload(&sc->light_pdf_dev, light_pdf.data(), light_pdf.size());
    if (e != cudaSuccess) return cuda_fail(e, "upload shading");
    sc->dev.shade = sc->shade;
    sc->dev.albedo = sc->albedo_dev;
    sc->dev.emission = sc->emission_dev;
    sc->dev.light_pdf = sc->light_pdf_dev;
    sc->dev.emissive = sc->emissive;
    sc->dev.emissive_cdf = sc->emissive_cdf;
    sc->dev.n_emissive = (int)em.size();
    sc->dev.emissive_total = (float)total;
    return DR_OK;
}

}  // namespace

extern "C" {

const char *dr_last_error(void) { return g_err.c_str(); }

int32_t dr_version(void) { return 200; }

int32_t dr_block_count(int32_t width, int32_t height) {
    if (width <= 0 || height <= 0) return 0;
    return ((width + DR_BLOCK_W - 1) / DR_BLOCK_W) * ((height + DR_BLOCK_H - 1) / DR_BLOCK_H);
}

// Lights::Spotlight constructor state (Spotlight.impl.cuh:5-33): colour x luminosity, normalised
// direction, emitter size at least 32 VECTOR_EPSILON, angles folded into [0, 180] with the falloff
// angle at least the hotspot angle (a negative falloff angle takes minus the hotspot angle, as the
// reference does), their cosines, 0..16 samples.
static void spotlight_state(const dr_light &l, drd::Light &d) {
    for (int k = 0; k < 3; k++) d.color[k] = l.color[k] * l.luminosity;
    float im = 1 / std::sqrt(l.direction[0] * l.direction[0] + l.direction[1] * l.direction[1] + l.direction[2] * l.direction[2]);
    for (int k = 0; k < 3; k++) d.direction[k] = l.direction[k] * im;
    const float eps = 0.000005f;
    d.emitter = (l.emitter_size < (32 * eps)) ? (32 * eps) : l.emitter_size;
    float inner = l.hotspot_angle, outer = l.falloff_angle;
    if (inner < 0.0f) inner = (-inner);
    if (inner > 180.0f) inner = 180.0f;
    if (outer < 0.0f) outer = (-inner);
    if (outer > 180.0f) outer = 180.0f;
    if (outer < inner) outer = inner;
    const float pi = 3.14159265359f;
    d.inner_cos = std::cos(inner * pi / 180.0f);
    d.outer_cos = std::cos(outer * pi / 180.0f);
    d.falloff = l.falloff_power;
    d.samples = (l.samples > 0) ? ((l.samples > 16) ? 16 : l.samples) : 0;
    d.shadows = l.cast_shadows ? 1 : 0;
    d.sphere = l.emit_from_sphere ? 1 : 0;
}

// Child boxes of every node group of T as planes of 8 (drd::Scene::gbox layout: 48 floats per group,
// lo x / y / z then hi x / y / z, 8 children each), in two versions.
static void group_planes(const drb::FlatOctree &T, std::vector<float> &gbox, std::vector<float> &gbox_ref) {
    //  * gbox_ref: the reference's boxes, except that an empty leaf's box is a point at kFar on every
    //    axis.  reduceNode has nothing to shrink an empty leaf to, so it keeps nearly its whole octant
    //    box, and on a displaced sphere the empty leaves hold about 2/3 of the leaves' surface area.
    //    An empty leaf yields no hit and adds to neither count of a cast (no triangles; the box-test
    //    count corrections follow the children taken on the way to a hit), and a ray reaches the far
    //    point only if its three slab distances to it coincide, when it just enters the empty leaf.
    //    The counting traversals of reference-padding scenes read these, so their counts are the
    //    reference's.
    //  * gbox: the boxes refitted to the non-empty leaves below (a leaf's own box; an inner node's
    //    union of its non-empty children's refitted boxes, empty subtrees at kFar).  The reference's
    //    inner boxes are unions that include the empty leaves' octant boxes; the refitted ones have
    //    about a third of their surface area.  A ray that misses a refitted box (the slab test's
    //    rounding is monotone in the box) misses every non-empty leaf box below it, so no leaf below
    //    could accept a hit: the visited leaves that matter, their order and every result are the
    //    reference's.  Every other traversal reads these.
    constexpr float kFar = 1e30f;
    const int64_t NN = T.node_count;
    const size_t groups = (size_t)(NN / 8);
    std::vector<float> fit_lo(3 * (size_t)NN), fit_hi(3 * (size_t)NN);
    std::vector<uint8_t> fit_live((size_t)NN, 0);
    auto refit_children = [&](int64_t first, float *lo, float *hi) {
        bool any = false;
        for (int k = 0; k < 3; k++) { lo[k] = kFar; hi[k] = -kFar; }
        for (int c = 0; c < 8; c++) {
            const int64_t j = first + c;
            if (!fit_live[j]) continue;
            any = true;
            for (int k = 0; k < 3; k++) {
                lo[k] = std::fmin(lo[k], fit_lo[3 * j + k]);
                hi[k] = std::fmax(hi[k], fit_hi[3 * j + k]);
            }
        }
        return any;
    };
    // node order is breadth-first (children after their parent), so reverse order is bottom-up
    for (int64_t i = NN - 1; i >= 0; i--) {
        if (T.node_child[i] < 0) {
            fit_live[i] = T.node_leaf_count[i] > 0;
            for (int k = 0; k < 3; k++) { fit_lo[3 * i + k] = T.node_lo[3 * i + k]; fit_hi[3 * i + k] = T.node_hi[3 * i + k]; }
        } else {
            fit_live[i] = refit_children(T.node_child[i], &fit_lo[3 * i], &fit_hi[3 * i]) ? 1 : 0;
        }
    }
    gbox.assign(48 * groups, 0.0f);
    gbox_ref.assign(48 * groups, 0.0f);
    for (size_t g = 0; g < groups; g++)
        for (int c = 0; c < 8; c++) {
            const int64_t j = 8 * (int64_t)g + c;
            const bool empty_leaf = T.node_child[j] < 0 && T.node_leaf_count[j] == 0;
            float *p = &gbox_ref[48 * g];
            for (int k = 0; k < 3; k++) {
                p[8 * k + c] = empty_leaf ? kFar : T.node_lo[3 * j + k];
                p[24 + 8 * k + c] = empty_leaf ? kFar : T.node_hi[3 * j + k];
            }
            float *q = &gbox[48 * g];
            for (int k = 0; k < 3; k++) {
                q[8 * k + c] = fit_live[j] ? fit_lo[3 * j + k] : kFar;
                q[24 + 8 * k + c] = fit_live[j] ? fit_hi[3 * j + k] : kFar;
            }
        }
}

dr_status dr_scene_create(const float *xyz, const float *nrm, const int32_t *mat_id, int32_t n, const dr_material *mats,
                          int32_t n_mats, const dr_light *lights, int32_t n_lights, const dr_build_params *bp, dr_scene **out) try {
    if (out == nullptr) return fail(DR_E_ARG, "dr_scene_create: out is NULL");
    *out = nullptr;
    if (n < 0 || (n > 0 && xyz == nullptr)) return fail(DR_E_ARG, "dr_scene_create: bad triangle array");
    if (n_mats < 0 || (n_mats > 0 && mats == nullptr)) return fail(DR_E_ARG, "dr_scene_create: bad material array");
    if (n_lights < 0 || (n_lights > 0 && lights == nullptr)) return fail(DR_E_ARG, "dr_scene_create: bad light array");
    if (n_lights > 16) return fail(DR_E_ARG, "dr_scene_create: at most 16 lights");
    for (int32_t i = 0; mat_id && i < n; i++)
        if (mat_id[i] < 0 || (n_mats > 0 && mat_id[i] >= n_mats) || (n_mats == 0 && mat_id[i] != 0))
            return fail(DR_E_ARG, "dr_scene_create: material id out of range at triangle " + std::to_string(i));
    for (int32_t i = 0; i < n_mats; i++) {
        if (mats[i].type < 0 || mats[i].type > DR_MAT_DEFAULT) return fail(DR_E_ARG, "dr_scene_create: bad material type");
        for (int k = 0; k < 4; k++)
            if (mats[i].texture[k] < 0) return fail(DR_E_ARG, "dr_scene_create: negative texture index");
    }
    for (int32_t i = 0; i < n_lights; i++)
        if (lights[i].type < 0 || lights[i].type > DR_LIGHT_SPOTLIGHT) return fail(DR_E_ARG, "dr_scene_create: bad light type");

    dr_scene *sc = new (std::nothrow) dr_scene();
    if (!sc) return fail(DR_E_NOMEM, "dr_scene_create: out of host memory");
    sc->n = n;
    sc->xyz.assign(xyz, xyz + 9 * (size_t)n);
    sc->mat_id.assign((size_t)n, 0);
    if (mat_id) std::copy(mat_id, mat_id + n, sc->mat_id.begin());
    sc->mats.assign(mats, mats + n_mats);

    drb::BuildOptions opt;
    if (bp) {
        if (bp->max_depth > 0) opt.max_depth = std::min(bp->max_depth, drd::kMaxDepth);
        if (bp->split_threshold > 0) opt.split_threshold = bp->split_threshold;
        opt.threads = bp->threads;
        opt.box_eps = bp->box_epsilon;
        opt.device = bp->device_build != 0;
    }
    std::string berr;
    if (!(opt.device ? drb::build_octree_gpu(sc->xyz.data(), n, opt, sc->tree, berr)
                     : drb::build_octree(sc->xyz.data(), n, opt, sc->tree))) {
        delete sc;
        return fail(opt.device ? DR_E_CUDA : DR_E_ARG, "dr_scene_create: octree build failed" + (berr.empty() ? std::string() : ": " + berr));
    }
    const drb::FlatOctree &T = sc->tree;
    if (T.node_count >= (int64_t(1) << 24)) {
        delete sc;
        return fail(DR_E_CAPACITY, "dr_scene_create: octree exceeds 2^24 nodes");
    }
    // pack nodes: {lo, first child | ~first ref}, {hi, ref count}
    std::vector<float4> nodes(2 * (size_t)T.node_count);
    for (int64_t i = 0; i < T.node_count; i++) {
        int w = T.node_child[i] >= 0 ? T.node_child[i] : ~(int)T.node_leaf_first[i];
        int c = T.node_child[i] >= 0 ? 0 : T.node_leaf_count[i];
        float wf, cf;
        std::memcpy(&wf, &w, 4);
        std::memcpy(&cf, &c, 4);
        nodes[2 * i] = make_float4(T.node_lo[3 * i], T.node_lo[3 * i + 1], T.node_lo[3 * i + 2], wf);
        nodes[2 * i + 1] = make_float4(T.node_hi[3 * i], T.node_hi[3 * i + 1], T.node_hi[3 * i + 2], cf);
    }
    std::vector<float4> leaf_tris(3 * T.leaf_refs.size());
    for (size_t r = 0; r < T.leaf_refs.size(); r++) {
        int id = T.leaf_refs[r];
        const float *p = &sc->xyz[9 * (size_t)id];
        float idf;
        std::memcpy(&idf, &id, 4);
        leaf_tris[3 * r] = make_float4(p[0], p[1], p[2], idf);
        leaf_tris[3 * r + 1] = make_float4(p[3], p[4], p[5], 0.0f);
        leaf_tris[3 * r + 2] = make_float4(p[6], p[7], p[8], 0.0f);
    }
    std::vector<float4> tris(3 * (size_t)n), nrms(3 * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const float *p = &sc->xyz[9 * i];
        for (int k = 0; k < 3; k++) tris[3 * i + k] = make_float4(p[3 * k], p[3 * k + 1], p[3 * k + 2], 0.0f);
        if (nrm) {
            const float *q = nrm + 9 * i;
            for (int k = 0; k < 3; k++) nrms[3 * i + k] = make_float4(q[3 * k], q[3 * k + 1], q[3 * k + 2], 0.0f);
        } else {
            float fn[3];
            flat_normal(p, fn);
            for (int k = 0; k < 3; k++) nrms[3 * i + k] = make_float4(fn[0], fn[1], fn[2], 0.0f);
        }
    }
    std::vector<drd::Material> dm(std::max(n_mats, 1));
    std::memset(dm.data(), 0, sizeof(drd::Material) * dm.size());
    for (int32_t i = 0; i < n_mats; i++) {
        const dr_material &m = mats[i];
        drd::Material &d = dm[i];
        d.type = m.type;
        for (int k = 0; k < 3; k++) { d.color[k] = m.color[k]; d.fresnel[k] = m.fresnel[k]; d.emission[k] = m.emission[k]; }
        d.specular = m.specular;
        d.metal = m.metal;
        d.diffuse = m.diffuse;
        d.smoothness = m.smoothness;
        d.shininess = m.shininess;
        d.roughness = m.roughness;
        for (int k = 0; k < 4; k++) {
            d.texture[k] = m.texture[k] - 1;
            d.tiling[k][0] = m.tiling[k][0];
            d.tiling[k][1] = m.tiling[k][1];
            d.offset[k][0] = m.offset[k][0];
            d.offset[k][1] = m.offset[k][1];
            sc->max_texture = std::max(sc->max_texture, m.texture[k]);
        }
        for (int k = 0; k < 3; k++) d.normal_color[k] = m.normal_color[k];
        d.alpha_threshold = m.alpha_threshold;
    }
    if (n_mats == 0) dm[0].type = DR_MAT_LAMBERT;
    std::vector<drd::Light> dl(std::max(n_lights, 1));
    std::memset(dl.data(), 0, sizeof(drd::Light) * dl.size());
    for (int32_t i = 0; i < n_lights; i++) {
        const dr_light &l = lights[i];
        drd::Light &d = dl[i];
        d.type = l.type;
        for (int k = 0; k < 3; k++) { d.color[k] = l.color[k]; d.position[k] = l.position[k]; d.direction[k] = l.direction[k]; }
        d.radius = l.radius;
        d.distance = l.distance;
        d.softness = l.softness;
        if (l.type == DR_LIGHT_SPOTLIGHT) spotlight_state(l, d);
    }

    std::vector<float> gbox, gbox_ref;
    group_planes(T, gbox, gbox_ref);
    float4 *d_nodes = nullptr, *d_gbox = nullptr, *d_gbox_ref = nullptr, *d_leaf = nullptr, *d_tris = nullptr, *d_nrms = nullptr;
    int *d_mat = nullptr;
    drd::Material *d_mats = nullptr;
    drd::Light *d_lights = nullptr;
    cudaError_t e = upload(&d_nodes, nodes.data(), nodes.size());
    if (e == cudaSuccess) { sc->allocs.push_back(d_nodes); e = upload(&d_gbox, (const float4 *)gbox.data(), gbox.size() / 4); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_gbox); e = upload(&d_gbox_ref, (const float4 *)gbox_ref.data(), gbox_ref.size() / 4); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_gbox_ref); e = upload(&d_leaf, leaf_tris.data(), leaf_tris.size()); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_leaf); e = upload(&d_tris, tris.data(), tris.size()); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_tris); e = upload(&d_nrms, nrms.data(), nrms.size()); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_nrms); e = upload(&d_mat, sc->mat_id.data(), sc->mat_id.size()); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_mat); e = upload(&d_mats, dm.data(), dm.size()); }
    if (e == cudaSuccess) { sc->allocs.push_back(d_mats); e = upload(&d_lights, dl.data(), dl.size()); }
    if (e == cudaSuccess) sc->allocs.push_back(d_lights);
    if (e != cudaSuccess) {
        delete sc;
        return cuda_fail(e, "dr_scene_create: upload");
    }
    sc->node_f4 = (int64_t)nodes.size();
    sc->leaf_f4 = (int64_t)leaf_tris.size();
    drd::Scene &S = sc->dev;
    S.nodes = d_nodes;
    S.gbox = d_gbox;
    S.gbox_ref = d_gbox_ref;
    S.leaf_tris = d_leaf;
    S.tris = d_tris;
    S.nrms = d_nrms;
    S.mat_id = d_mat;
    S.mats = d_mats;
    S.lights = d_lights;
    for (int k = 0; k < 3; k++) { S.root_lo[k] = T.root_lo[k]; S.root_hi[k] = T.root_hi[k]; }
    S.root_child = T.root_child >= 0 ? 0 : -1;
    S.root_leaf_first = (int)T.root_leaf_first;
    S.root_leaf_count = T.root_leaf_count;
    S.n_tris = n;
    S.front_only = (bp && bp->box_epsilon != 0.0f) ? 1 : 0;
    S.n_mats = std::max(n_mats, 1);
    S.n_lights = n_lights;
    S.shadow_photons = 0;
    for (int32_t i = 0; i < n_lights; i++)
        S.shadow_photons += (lights[i].type == DR_LIGHT_SPOTLIGHT) ? (dl[i].shadows ? dl[i].samples : 0) : 1;
    if (n == 0) { S.root_child = -1; S.root_leaf_count = 0; }

    sc->albedo.resize(3 * (size_t)n);
    sc->emission.resize(3 * (size_t)n);
    sc->roughness.resize((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const drd::Material &m = dm[sc->mat_id[i]];
        for (int k = 0; k < 3; k++) { sc->albedo[3 * i + k] = m.color[k]; sc->emission[3 * i + k] = m.emission[k]; }
        sc->roughness[i] = m.roughness;
    }
    dr_status st = upload_shading(sc);
    if (st != DR_OK) { delete sc; return st; }
    *out = sc;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_create");
}

dr_status dr_scene_set_triangle_params(dr_scene *sc, const float *albedo, const float *emission, const float *roughness) try {
    if (!sc) return fail(DR_E_ARG, "dr_scene_set_triangle_params: scene is NULL");
    size_t n = (size_t)sc->n;
    if (albedo) std::copy(albedo, albedo + 3 * n, sc->albedo.begin());
    if (emission) std::copy(emission, emission + 3 * n, sc->emission.begin());
    if (roughness) std::copy(roughness, roughness + n, sc->roughness.begin());
    return upload_shading(sc);
} catch (...) {
    return dr_internal_exception("dr_scene_set_triangle_params");
}

dr_status dr_scene_set_textures(dr_scene *sc, const dr_texture *tex, int32_t n, const float *uv) try {
    if (!sc || n < 0 || (n > 0 && !tex)) return fail(DR_E_ARG, "dr_scene_set_textures: bad arguments");
    if (sc->max_texture > n) return fail(DR_E_ARG, "dr_scene_set_textures: a material uses texture " +
                                                       std::to_string(sc->max_texture) + " of " + std::to_string(n));
    std::vector<float4> texels;
    std::vector<int4> info;
    for (int32_t t = 0; t < n; t++) {
        const dr_texture &x = tex[t];
        if (x.width <= 0 || x.height <= 0 || !x.rgba || (x.filtering != DR_FILTER_NONE && x.filtering != DR_FILTER_BILINEAR))
            return fail(DR_E_ARG, "dr_scene_set_textures: bad texture " + std::to_string(t));
        const size_t texel_count = (size_t)x.width * (size_t)x.height;
        if (texels.size() + texel_count > (size_t)INT32_MAX) return fail(DR_E_ARG, "dr_scene_set_textures: too many texels");
        info.push_back(make_int4((int)texels.size(), x.width, x.height, x.filtering));
        for (size_t k = 0; k < texel_count; k++)
            texels.push_back(make_float4(x.rgba[4 * k], x.rgba[4 * k + 1], x.rgba[4 * k + 2], x.rgba[4 * k + 3]));
    }
    std::vector<float2> uv2((size_t)3 * (size_t)std::max<int64_t>(sc->n, 1), make_float2(0.0f, 0.0f));
    if (uv)
        for (int64_t i = 0; i < 3 * sc->n; i++) uv2[(size_t)i] = make_float2(uv[2 * i], uv[2 * i + 1]);
    float4 *d_texels = nullptr;
    int4 *d_info = nullptr;
    float2 *d_uv = nullptr;
    cudaError_t e = cudaSuccess;
    if (!texels.empty()) e = upload(&d_texels, texels.data(), texels.size());
    if (e == cudaSuccess && !info.empty()) e = upload(&d_info, info.data(), info.size());
    if (e == cudaSuccess) e = upload(&d_uv, uv2.data(), uv2.size());
    if (e != cudaSuccess) {
        cudaFree(d_texels);
        cudaFree(d_info);
        cudaFree(d_uv);
        return cuda_fail(e, "dr_scene_set_textures");
    }
    // replaced buffers stay allocated until the scene is destroyed: batches created earlier hold
    // copies of the scene's device view
    for (void *old : {(void *)sc->texels_dev, (void *)sc->tex_info_dev, (void *)sc->uv_dev})
        if (old) sc->allocs.push_back(old);
    sc->texels_dev = d_texels;
    sc->tex_info_dev = d_info;
    sc->uv_dev = d_uv;
    sc->n_textures = n;
    sc->dev.texels = d_texels;
    sc->dev.tex_info = d_info;
    sc->dev.uv = d_uv;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_set_textures");
}

dr_status dr_scene_triangle_params_device(dr_scene *sc, float **albedo, float **emission) try {
    if (!sc) return fail(DR_E_ARG, "dr_scene_triangle_params_device: scene is NULL");
    if (albedo) *albedo = sc->albedo_dev;
    if (emission) *emission = sc->emission_dev;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_triangle_params_device");
}

static void tree_stats(const drb::FlatOctree &T, int64_t *nodes, int64_t *leaves, int64_t *refs, int32_t *depth) {
    int64_t nl = (T.root_child < 0) ? 1 : 0;
    for (int64_t i = 0; i < T.node_count; i++) nl += (T.node_child[i] < 0) ? 1 : 0;
    if (nodes) *nodes = T.node_count + 1;
    if (leaves) *leaves = nl;
    if (refs) *refs = (int64_t)T.leaf_refs.size();
    if (depth) *depth = T.depth;
}

static void tree_export(const drb::FlatOctree &T, float *node_box, int32_t *node_child, int32_t *node_leaf, int32_t *leaf_tri) {
    // node 0 = root, node i + 1 = flat node i
    auto put = [&](int64_t at, const float *lo, const float *hi, int32_t child, int64_t first, int32_t count) {
        if (node_box) {
            for (int k = 0; k < 3; k++) { node_box[6 * at + k] = lo[k]; node_box[6 * at + 3 + k] = hi[k]; }
        }
        if (node_child) node_child[at] = child;
        if (node_leaf) {
            node_leaf[2 * at] = child >= 0 ? 0 : (int32_t)first;
            node_leaf[2 * at + 1] = child >= 0 ? 0 : count;
        }
    };
    put(0, T.root_lo, T.root_hi, T.root_child >= 0 ? 1 : -1, T.root_leaf_first, T.root_leaf_count);
    for (int64_t i = 0; i < T.node_count; i++)
        put(i + 1, &T.node_lo[3 * i], &T.node_hi[3 * i], T.node_child[i] >= 0 ? T.node_child[i] + 1 : -1, T.node_leaf_first[i],
            T.node_leaf_count[i]);
    if (leaf_tri) std::copy(T.leaf_refs.begin(), T.leaf_refs.end(), leaf_tri);
}

dr_status dr_scene_stats(const dr_scene *sc, int64_t *nodes, int64_t *leaves, int64_t *refs, int32_t *depth) try {
    if (!sc) return fail(DR_E_ARG, "dr_scene_stats: scene is NULL");
    tree_stats(sc->tree, nodes, leaves, refs, depth);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_stats");
}

dr_status dr_scene_export_tree(const dr_scene *sc, float *node_box, int32_t *node_child, int32_t *node_leaf, int32_t *leaf_tri) try {
    if (!sc) return fail(DR_E_ARG, "dr_scene_export_tree: scene is NULL");
    tree_export(sc->tree, node_box, node_child, node_leaf, leaf_tri);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_export_tree");
}

dr_status dr_octree_create_host(const float *xyz, int32_t n, const dr_build_params *bp, dr_octree **out) try {
    if (!out) return fail(DR_E_ARG, "dr_octree_create_host: out is NULL");
    *out = nullptr;
    if (n < 0 || (n > 0 && !xyz)) return fail(DR_E_ARG, "dr_octree_create_host: bad triangle array");
    dr_octree *t = new (std::nothrow) dr_octree();
    if (!t) return fail(DR_E_NOMEM, "dr_octree_create_host: out of host memory");
    drb::BuildOptions opt;
    if (bp) {
        if (bp->max_depth > 0) opt.max_depth = std::min(bp->max_depth, drd::kMaxDepth);
        if (bp->split_threshold > 0) opt.split_threshold = bp->split_threshold;
        opt.threads = bp->threads;
        opt.box_eps = bp->box_epsilon;
        opt.device = bp->device_build != 0;
    }
    std::string berr;
    if (!(opt.device ? drb::build_octree_gpu(xyz, n, opt, t->tree, berr) : drb::build_octree(xyz, n, opt, t->tree))) {
        delete t;
        return fail(opt.device ? DR_E_CUDA : DR_E_ARG, "dr_octree_create_host: build failed" + (berr.empty() ? std::string() : ": " + berr));
    }
    *out = t;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_octree_create_host");
}

dr_status dr_octree_stats(const dr_octree *t, int64_t *nodes, int64_t *leaves, int64_t *refs, int32_t *depth) try {
    if (!t) return fail(DR_E_ARG, "dr_octree_stats: tree is NULL");
    tree_stats(t->tree, nodes, leaves, refs, depth);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_octree_stats");
}

dr_status dr_octree_export(const dr_octree *t, float *node_box, int32_t *node_child, int32_t *node_leaf, int32_t *leaf_tri) try {
    if (!t) return fail(DR_E_ARG, "dr_octree_export: tree is NULL");
    tree_export(t->tree, node_box, node_child, node_leaf, leaf_tri);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_octree_export");
}

dr_status dr_octree_group_planes(const dr_octree *t, float *gbox, float *gbox_ref) try {
    if (!t) return fail(DR_E_ARG, "dr_octree_group_planes: tree is NULL");
    std::vector<float> g, r;
    group_planes(t->tree, g, r);
    if (gbox && !g.empty()) std::memcpy(gbox, g.data(), sizeof(float) * g.size());
    if (gbox_ref && !r.empty()) std::memcpy(gbox_ref, r.data(), sizeof(float) * r.size());
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_octree_group_planes");
}

void dr_octree_destroy(dr_octree *t) { delete t; }

void dr_scene_destroy(dr_scene *sc) { delete sc; }

static dr_status cast_impl(const dr_scene *sc, const float *o, const float *d, const int32_t *ignore, int32_t n, int32_t clip,
                           int32_t *hit_tri, float *hit_t, int32_t *nbox, int32_t *ntri, void *stream) {
    if (!sc) return fail(DR_E_ARG, "dr_cast: scene is NULL");
    if (n < 0) return fail(DR_E_ARG, "dr_cast: negative ray count");
    if (n == 0) return DR_OK;
    if (!o || !d || !hit_tri || !hit_t) return fail(DR_E_ARG, "dr_cast: NULL buffer");
    cudaError_t e = drk::launch_cast(sc->dev, o, d, ignore, n, clip, hit_tri, hit_t, nbox, ntri, (cudaStream_t)stream, nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "dr_cast");
    return DR_OK;
}

dr_status dr_cast(const dr_scene *sc, const float *o, const float *d, const int32_t *ignore, int32_t n, int32_t clip,
                  int32_t *hit_tri, float *hit_t, void *stream) try {
    return cast_impl(sc, o, d, ignore, n, clip, hit_tri, hit_t, nullptr, nullptr, stream);
} catch (...) {
    return dr_internal_exception("dr_cast");
}

dr_status dr_cast_counted(const dr_scene *sc, const float *o, const float *d, const int32_t *ignore, int32_t n, int32_t clip,
                          int32_t *hit_tri, float *hit_t, int32_t *nbox, int32_t *ntri, void *stream) try {
    if (!nbox || !ntri) return fail(DR_E_ARG, "dr_cast_counted: NULL counter buffer");
    return cast_impl(sc, o, d, ignore, n, clip, hit_tri, hit_t, nbox, ntri, stream);
} catch (...) {
    return dr_internal_exception("dr_cast_counted");
}

dr_status dr_renderer_create(int32_t wave_paths, dr_renderer **out) try {
    if (!out) return fail(DR_E_ARG, "dr_renderer_create: out is NULL");
    *out = nullptr;
    if (wave_paths < 0) return fail(DR_E_ARG, "dr_renderer_create: negative wave size");
    if (wave_paths == 0) wave_paths = 1 << 22;
    wave_paths = ((wave_paths + 31) / 32) * 32;
    dr_renderer *r = new (std::nothrow) dr_renderer();
    if (!r) return fail(DR_E_NOMEM, "dr_renderer_create: out of host memory");
    r->capacity = wave_paths;
    r->shadow_capacity = wave_paths * 2;
    r->lanes = DR_DEFAULT_LANES;
    size_t W = (size_t)wave_paths;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        for (int j = 0; j < 3 && e == cudaSuccess; j++) e = cudaMalloc((void **)&r->q[k][j], sizeof(float4) * W);
        if (e == cudaSuccess) e = cudaMalloc((void **)&r->q3[k], sizeof(int4) * W);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&r->hits, sizeof(float2) * W);
    for (int j = 0; j < 5 && e == cudaSuccess; j++)
        e = cudaMalloc((void **)&r->s[j], sizeof(float4) * drd::shadow_plane_records(r->shadow_capacity));
    if (e == cudaSuccess) e = cudaMalloc(&r->ctrl, drk::ctrl_bytes());
    if (e != cudaSuccess) {
        delete r;
        return cuda_fail(e, "dr_renderer_create");
    }
    *out = r;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_create");
}

void dr_renderer_destroy(dr_renderer *r) { delete r; }

int64_t dr_renderer_launch_count(const dr_renderer *r) { return r ? r->launches : 0; }

dr_status dr_renderer_set_profiling(dr_renderer *r, int32_t enable) try {
    if (!r) return fail(DR_E_ARG, "dr_renderer_set_profiling: renderer is NULL");
    r->prof.reset(enable != 0);
    r->prof.enabled = enable != 0;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_set_profiling");
}

dr_status dr_renderer_kernel_busy(dr_renderer *r, double *busy_ms) try {
    if (!r || !busy_ms) return fail(DR_E_ARG, "dr_renderer_kernel_busy: NULL argument");
    cudaError_t e = r->prof.harvest();
    if (e != cudaSuccess) return cuda_fail(e, "dr_renderer_kernel_busy");
    r->prof.busy(busy_ms);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_kernel_busy");
}

dr_status dr_renderer_set_lanes(dr_renderer *r, int32_t lanes) try {
    if (!r) return fail(DR_E_ARG, "dr_renderer_set_lanes: renderer is NULL");
    if (lanes < 1 || lanes > DR_MAX_LANES) return fail(DR_E_ARG, "dr_renderer_set_lanes: lanes must be in [1, 8]");
    r->lanes = lanes;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_set_lanes");
}

int32_t dr_renderer_lanes(const dr_renderer *r) { return r ? r->lanes : 0; }

dr_status dr_renderer_set_block_shape(dr_renderer *r, int32_t shape) try {
    if (!r) return fail(DR_E_ARG, "dr_renderer_set_block_shape: renderer is NULL");
    if (shape < 0 || shape > 1) return fail(DR_E_ARG, "dr_renderer_set_block_shape: shape must be 0 or 1");
    r->shape = shape;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_set_block_shape");
}

int32_t dr_renderer_block_shape(const dr_renderer *r) { return r ? r->shape : -1; }

dr_status dr_renderer_kernel_times(dr_renderer *r, double *ms, int64_t *launches) try {
    if (!r) return fail(DR_E_ARG, "dr_renderer_kernel_times: renderer is NULL");
    cudaError_t e = r->prof.harvest();
    if (e != cudaSuccess) return cuda_fail(e, "dr_renderer_kernel_times");
    for (int k = 0; k < DR_KERNEL_CLASSES; k++) {
        if (ms) ms[k] = r->prof.ms[k];
        if (launches) launches[k] = r->prof.launches[k];
    }
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_kernel_times");
}

dr_status dr_renderer_set_counting(dr_renderer *r, int32_t enable) try {
    if (!r) return fail(DR_E_ARG, "dr_renderer_set_counting: renderer is NULL");
    if (!r->counters) {
        cudaError_t e = cudaMalloc((void **)&r->counters, 6 * sizeof(unsigned long long));
        if (e != cudaSuccess) return cuda_fail(e, "dr_renderer_set_counting");
    }
    cudaError_t e = cudaMemset(r->counters, 0, 6 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "dr_renderer_set_counting");
    r->counting = enable != 0;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_set_counting");
}

dr_status dr_renderer_wave_counts(dr_renderer *r, int32_t *rays, int32_t *shadow_records, int32_t n) try {
    if (!r || !rays || !shadow_records) return fail(DR_E_ARG, "dr_renderer_wave_counts: NULL argument");
    if (n < 0 || n > drd::kMaxBounceSlots) return fail(DR_E_ARG, "dr_renderer_wave_counts: n must be in [0, 68]");
    if (n == 0) return DR_OK;
    if (!r->ctrl) return fail(DR_E_STATE, "dr_renderer_wave_counts: the renderer has not rendered");
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = drk::read_wave_counts(r->ctrl, rays, shadow_records, n);
    if (e != cudaSuccess) return cuda_fail(e, "dr_renderer_wave_counts");
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_wave_counts");
}

dr_status dr_renderer_counters(dr_renderer *r, int64_t *counts) try {
    if (!r || !counts) return fail(DR_E_ARG, "dr_renderer_counters: NULL argument");
    unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
    if (r->counters) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(h, r->counters, sizeof(h), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "dr_renderer_counters");
    }
    for (int k = 0; k < 6; k++) counts[k] = (int64_t)h[k];
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_renderer_counters");
}

}  // extern "C"

// Validates one render job and fills its Item (everything but the slot / path offsets).  Shared by
// dr_render_blocks, the batch builder and dr_render_blocks_noalloc (declared in dr_internal.h).
dr_status dr_internal_make_item(const dr_scene *sc, const dr_camera *cam, float *fb, int32_t start_block,
                                int32_t end_block, const dr_render_params *p, const char *who, drk::Item &I) {
    if (!sc || !cam || !fb || !p) return fail(DR_E_ARG, std::string(who) + ": NULL argument");
    if (sc->max_texture > sc->n_textures)
        return fail(DR_E_ARG, std::string(who) + ": the scene's materials use textures it does not have (dr_scene_set_textures)");
    if (p->mode != DR_MODE_REFERENCE && p->mode != DR_MODE_PHYSICAL) return fail(DR_E_ARG, std::string(who) + ": bad mode");
    if (p->width <= 0 || p->height <= 0) return fail(DR_E_ARG, std::string(who) + ": bad resolution");
    const int nblocks = dr_block_count(p->width, p->height);
    if (start_block < 0 || end_block > nblocks || start_block > end_block)
        return fail(DR_E_ARG, std::string(who) + ": bad block range");
    if (p->max_bounces < 0 || p->max_bounces > 64) return fail(DR_E_ARG, std::string(who) + ": max_bounces must be in [0, 64]");
    if (p->boxing < 0 || p->boxing > 3) return fail(DR_E_ARG, std::string(who) + ": bad boxing mode");
    if (cam->lens < 0 || cam->lens > DR_LENS_SPHERICAL) return fail(DR_E_ARG, std::string(who) + ": bad lens");
    if ((p->mode == DR_MODE_REFERENCE) != (cam->lens <= DR_LENS_SPHERICAL_SEGMENT))
        return fail(DR_E_ARG, std::string(who) + ": lens does not belong to the render mode");
    const int fx = std::max(1, p->samples_x), fy = std::max(1, p->samples_y);
    std::memset(&I, 0, sizeof(I));
    I.S = sc->dev;
    I.camera = *cam;
    {
        float angle = cam->angle[0];
        if (angle < 1.0f) angle = 1.0f;
        else if (angle > 179.0f) angle = 179.0f;
        float radian = (angle / (2 * 57.29577951308233f));
        I.cam_x = (cam->lens_x > 0.0f) ? cam->lens_x : 0.5f / std::tan(radian);
    }
    I.mode = p->mode;
    I.width = p->width;
    I.height = p->height;
    I.fsaa_x = fx;
    I.fsaa_y = fy;
    I.spp = fx * fy;
    I.max_bounces = p->max_bounces;
    I.clip = p->cull_backfaces;
    {
        float w = (float)p->width, h = (float)p->height;
        float ps;
        if (p->boxing == DR_BOXING_HEIGHT) ps = 1.0f / h;
        else if (p->boxing == DR_BOXING_WIDTH) ps = 1.0f / w;
        else if (p->boxing == DR_BOXING_MIN) ps = 1.0f / ((h <= w) ? h : w);
        else ps = 1.0f / ((h >= w) ? h : w);
        I.pixel_size = ps;
        I.pdx = ps / (float)fx;
        I.pdy = ps / (float)fy;
    }
    I.seed = p->seed;
    I.sample_base = (uint32_t)((p->iteration < 1 ? 0 : p->iteration - 1) * I.spp);
    I.start_block = start_block;
    I.n_slots = (end_block - start_block) * DR_BLOCK_W * DR_BLOCK_H;
    I.fb = fb;
    I.inv_spp = 1.0f / (float)I.spp;
    I.blend = (p->iteration <= 1) ? 1.0f : (1.0f / (float)p->iteration);
    return DR_OK;
}

extern "C" {

static dr_status ensure_accum(dr_renderer *r, size_t slots) {
    if (r->accum_slots >= slots) return DR_OK;
    cudaFree(r->accum);
    r->accum = nullptr;
    r->accum_slots = 0;
    cudaError_t e = cudaMalloc((void **)&r->accum, sizeof(float4) * std::max<size_t>(slots, 1));
    if (e != cudaSuccess) return cuda_fail(e, "accumulator");
    r->accum_slots = slots;
    r->scratch_id = dr_renderer::next_scratch_id();
    return DR_OK;
}

static void wave_buffers(dr_renderer *r, drk::WaveDesc &W) {
    for (int k = 0; k < 2; k++) {
        W.q_p0[k] = r->q[k][0];
        W.q_p1[k] = r->q[k][1];
        W.q_p2[k] = r->q[k][2];
        W.q_p3[k] = r->q3[k];
    }
    W.hits = r->hits;
    for (int j = 0; j < 5; j++) W.s[j] = r->s[j];
    W.shadow_cap = r->shadow_capacity;
    W.accum = r->accum;
    W.ctrl = r->ctrl;
    W.prefix = r->prefix;
    W.shape = r->shape;
}

// Wave size for `lanes` concurrent pipelines: at most `wave`, and small enough that a render of
// `total` paths splits into about `lanes` balanced waves, but not below kMinLaneWave paths (smaller
// waves cannot fill the GPU; such renders keep fewer lanes).
constexpr long long kMinLaneWave = 1 << 18;
static long long lane_wave(long long total, long long wave, int lanes) {
    if (lanes <= 1) return wave;
    long long w = (total + lanes - 1) / lanes;
    w = std::max<long long>(w, kMinLaneWave);
    w = ((w + 31) / 32) * 32;
    return std::min<long long>(wave, w);
}

// Lanes a render of `total` paths in waves of `wave` uses: no more than it has waves.
static int lanes_used(long long total, long long wave, int lanes) {
    const long long n_waves = (total + wave - 1) / wave;
    return (int)std::max<long long>(1, std::min<long long>(lanes, n_waves));
}

// Allocates the renderer's extra lanes up to `n` (same wave capacity as the renderer).
static dr_status ensure_lanes(dr_renderer *r, int n) {
    cudaError_t e = cudaSuccess;
    if (!r->fork) e = cudaEventCreateWithFlags(&r->fork, cudaEventDisableTiming);
    while (e == cudaSuccess && (int)r->extra.size() < n) {
        WaveScratch l;
        e = l.alloc((size_t)r->capacity, (size_t)r->shadow_capacity);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            l.release();
            break;
        }
        r->extra.push_back(l);
    }
    if (e != cudaSuccess) return cuda_fail(e, "render: lane scratch");
    return DR_OK;
}

// Issues the waves (and the resolve unless adjoint) of `total` paths over `total_slots` slots.
// With lanes > 1, wave i runs on lane i % lanes: lane 0 is the renderer's own scratch on `stream`,
// the others fork from and join back into `stream` through events.
static dr_status run_waves(dr_renderer *r, drk::WaveDesc &W, long long total, long long wave, int total_slots, cudaStream_t stream,
                           drk::Profiler *prof, bool count, bool resolve, int lanes = 1) {
    cudaError_t e = cudaMemsetAsync(r->accum, 0, sizeof(float4) * (size_t)std::max(total_slots, 1), stream);
    if (e != cudaSuccess) return cuda_fail(e, "render: clear accumulator");
    const int L = lanes_used(total, wave, lanes);
    if (L > 1) {
        dr_status st = ensure_lanes(r, L - 1);
        if (st != DR_OK) return st;
        e = cudaEventRecord(r->fork, stream);
        for (int k = 0; k < L - 1 && e == cudaSuccess; k++) e = cudaStreamWaitEvent(r->extra[k].stream, r->fork, 0);
        if (e != cudaSuccess) return cuda_fail(e, "render: fork lanes");
    }
    long long i = 0;
    for (long long b = 0; b < total; b += wave, i++) {
        const int l = (int)(i % L);
        drk::WaveDesc Wl = W;
        cudaStream_t sl = stream;
        if (l > 0) {
            const WaveScratch &x = r->extra[l - 1];
            for (int k = 0; k < 2; k++) {
                Wl.q_p0[k] = x.q[k][0];
                Wl.q_p1[k] = x.q[k][1];
                Wl.q_p2[k] = x.q[k][2];
                Wl.q_p3[k] = x.q3[k];
            }
            Wl.hits = x.hits;
            for (int j = 0; j < 5; j++) Wl.s[j] = x.s[j];
            Wl.ctrl = x.ctrl;
            Wl.prefix = x.prefix;
            sl = x.stream;
        }
        Wl.wave_begin = b;
        Wl.wave_count = (int)std::min<long long>(wave, total - b);
        e = drk::launch_wave(Wl, sl, &r->launches, prof, count ? r->counters : nullptr);
        if (e != cudaSuccess) return cuda_fail(e, "render: wave");
    }
    if (L > 1) {
        for (int k = 0; k < L - 1 && e == cudaSuccess; k++) {
            e = cudaEventRecord(r->extra[k].done, r->extra[k].stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, r->extra[k].done, 0);
        }
        if (e != cudaSuccess) return cuda_fail(e, "render: join lanes");
    }
    if (resolve) {
        e = drk::launch_resolve(W, total_slots, stream, &r->launches, prof);
        if (e != cudaSuccess) return cuda_fail(e, "render: resolve");
    }
    return DR_OK;
}

// An adjoint lane's prefix buffer: kAdjDepth triangle indices per path of a wave.
static cudaError_t ensure_prefix(int *&prefix, int &paths, long long wave) {
    if (paths >= wave) return cudaSuccess;
    cudaFree(prefix);
    prefix = nullptr;
    paths = 0;
    cudaError_t e = cudaMalloc((void **)&prefix, sizeof(int) * (size_t)wave * drd::kAdjDepth);
    if (e == cudaSuccess) paths = (int)wave;
    return e;
}

static long long wave_size(const dr_renderer *r, int lights_per_path, long long cap) {
    long long wave = std::min<long long>(std::min<long long>(r->capacity, cap), (long long)r->shadow_capacity / std::max(1, lights_per_path));
    return std::max<long long>(32, (wave / 32) * 32);
}

dr_status dr_render_blocks(dr_renderer *r, const dr_scene *sc, const dr_camera *cam, float *fb, int32_t start_block,
                           int32_t end_block, const dr_render_params *p, void *stream_ptr) try {
    if (!r) return fail(DR_E_ARG, "dr_render_blocks: NULL argument");
    drk::WaveDesc W;
    std::memset(&W, 0, sizeof(W));
    dr_status st = dr_internal_make_item(sc, cam, fb, start_block, end_block, p, "dr_render_blocks", W.inl);
    if (st != DR_OK) return st;
    if (start_block == end_block) return DR_OK;
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    const drk::Item &I = W.inl;
    st = ensure_accum(r, (size_t)I.n_slots);
    if (st != DR_OK) return st;
    W.items = nullptr;
    W.n_items = 1;
    W.mode = I.mode;
    W.max_bounces = I.max_bounces;
    W.adjoint = false;
    wave_buffers(r, W);
    const int lights = (I.mode == DR_MODE_REFERENCE) ? I.S.shadow_photons : 1;
    const long long total = (long long)I.n_slots * I.spp;
    const long long wave = lane_wave(total, wave_size(r, lights, 1LL << 40), r->lanes);
    return run_waves(r, W, total, wave, I.n_slots, stream, &r->prof, r->counting, true, r->lanes);
} catch (...) {
    return dr_internal_exception("dr_render_blocks");
}

dr_status dr_render_adjoint(dr_renderer *r, const dr_scene *sc, const dr_camera *cam, const float *dl_dfb, int32_t start_block,
                            int32_t end_block, const dr_render_params *p, float *grad_albedo, float *grad_emission,
                            void *stream_ptr) try {
    if (!r || !dl_dfb || !grad_albedo || !grad_emission) return fail(DR_E_ARG, "dr_render_adjoint: NULL argument");
    drk::WaveDesc W;
    std::memset(&W, 0, sizeof(W));
    dr_status st = dr_internal_make_item(sc, cam, const_cast<float *>(dl_dfb), start_block, end_block, p, "dr_render_adjoint", W.inl);
    if (st != DR_OK) return st;
    if (p->mode != DR_MODE_PHYSICAL) return fail(DR_E_ARG, "dr_render_adjoint: only the physical mode is differentiable");
    if (p->max_bounces + 1 > drd::kAdjDepth) return fail(DR_E_ARG, "dr_render_adjoint: too many bounces");
    if (start_block == end_block) return DR_OK;
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    drk::Item &I = W.inl;
    I.fb = nullptr;
    I.dl_dfb = dl_dfb;
    I.grad_albedo = grad_albedo;
    I.grad_emission = grad_emission;
    const long long cap = 1LL << 20;  // paths per adjoint wave: bounds each lane's prefix buffer to ~280 MB
    const long long total = (long long)I.n_slots * I.spp;
    const long long wave = lane_wave(total, wave_size(r, 1, cap), r->lanes);
    const int L = lanes_used(total, wave, r->lanes);
    if (L > 1) {
        st = ensure_lanes(r, L - 1);
        if (st != DR_OK) return st;
    }
    cudaError_t e = ensure_prefix(r->prefix, r->prefix_paths, wave);
    for (int k = 0; k < L - 1 && e == cudaSuccess; k++) e = ensure_prefix(r->extra[k].prefix, r->extra[k].prefix_paths, wave);
    if (e != cudaSuccess) return cuda_fail(e, "dr_render_adjoint: prefix buffer");
    st = ensure_accum(r, (size_t)I.n_slots);
    if (st != DR_OK) return st;
    W.items = nullptr;
    W.n_items = 1;
    W.mode = I.mode;
    W.max_bounces = I.max_bounces;
    W.adjoint = true;
    wave_buffers(r, W);
    return run_waves(r, W, total, wave, I.n_slots, stream, &r->prof, false, false, L);
} catch (...) {
    return dr_internal_exception("dr_render_adjoint");
}

}  // extern "C"

// ---- batches ------------------------------------------------------------------------------------
struct dr_batch {
    std::vector<drk::Item> items;
    drk::Item *items_dev = nullptr;
    long long total_paths = 0;
    int total_slots = 0;
    int mode = 0, max_bounces = 0, max_lights = 1;
    std::vector<const dr_scene *> scenes;
    std::vector<dr_render_params> params;
    unsigned long long graph_scratch = 0;   // scratch_id of the renderer the graph was captured with
    long long graph_wave = 0;
    int graph_lanes = 0;
    int graph_shape = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graph_launches = 0;
    // Captures run on this private stream: the caller's stream may be the legacy default stream,
    // which cannot be captured.  The instantiated graph is launched on the caller's stream.
    cudaStream_t capture_stream = nullptr;
    cudaEvent_t done = nullptr;   // recorded after each render: the job table is in use until it fires
    // One device arena holding the octrees of all the batch's scenes (node child / leaf indices
    // rebased), so the traversal reads nodes and leaf triangles through one pointer for every ray.
    float4 *arena_nodes = nullptr, *arena_gbox = nullptr, *arena_leaf = nullptr;
    int64_t arena_node_count = 0;

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        graph_scratch = 0;
    }
    ~dr_batch() {
        drop_graph();
        if (capture_stream) cudaStreamDestroy(capture_stream);
        if (done) cudaEventDestroy(done);
        cudaFree(arena_nodes);
        cudaFree(arena_gbox);
        cudaFree(arena_leaf);
        cudaFree(items_dev);
    }
};

extern "C" {

// Concatenates the octrees of the batch's distinct scenes into one device arena and points every
// job's scene record at it: node groups and leaf records of scene k start after those of scenes
// 0..k-1; triangle ids in the leaf records stay scene-local (a ray only visits its own scene's nodes).
static dr_status build_arena(dr_batch *b) {
    std::vector<const dr_scene *> uniq;
    std::vector<int64_t> node_off, leaf_off;
    int64_t nodes = 0, leaf = 0;
    for (const dr_scene *sc : b->scenes) {
        if (std::find(uniq.begin(), uniq.end(), sc) != uniq.end()) continue;
        if ((sc->node_f4 / 2) % 8 != 0) return fail(DR_E_STATE, "dr_batch_create: octree nodes are not in groups of 8");
        uniq.push_back(sc);
        node_off.push_back(nodes / 2);
        leaf_off.push_back(leaf / 3);
        nodes += sc->node_f4;
        leaf += sc->leaf_f4;
    }
    b->arena_node_count = nodes / 2;
    if (b->arena_node_count >= (int64_t(1) << 27) || leaf / 3 >= (int64_t(1) << 31))
        return fail(DR_E_CAPACITY, "dr_batch_create: the scenes' octrees exceed 2^27 nodes or 2^31 leaf references");
    cudaError_t e = cudaMalloc((void **)&b->arena_nodes, sizeof(float4) * (size_t)std::max<int64_t>(nodes, 2));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->arena_leaf, sizeof(float4) * (size_t)std::max<int64_t>(leaf, 3));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->arena_gbox, sizeof(float4) * 12 * (size_t)std::max<int64_t>(nodes / 16, 1));
    for (size_t k = 0; k < uniq.size() && e == cudaSuccess; k++) {
        const dr_scene *sc = uniq[k];
        if (sc->leaf_f4)
            e = cudaMemcpy(b->arena_leaf + 3 * leaf_off[k], sc->dev.leaf_tris, sizeof(float4) * (size_t)sc->leaf_f4,
                           cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess && sc->node_f4)
            e = cudaMemcpy(b->arena_gbox + 12 * (node_off[k] / 8), sc->dev.gbox, sizeof(float4) * 12 * (size_t)(sc->node_f4 / 16),
                           cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess && sc->node_f4)
            e = drk::launch_rebase_nodes(b->arena_nodes + 2 * node_off[k], sc->dev.nodes, sc->node_f4 / 2, (int)(node_off[k] / 8),
                                         (int)leaf_off[k], nullptr);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "dr_batch_create: octree arena");
    // the traversal reads the behind-origin culling flag from the arena (uniform): on only if every
    // scene of the batch allows it
    int front = 1;
    for (const dr_scene *sc : uniq) front &= sc->dev.front_only;
    for (size_t i = 0; i < b->items.size(); i++) {
        b->items[i].S.front_only = front;
        const size_t k = (size_t)(std::find(uniq.begin(), uniq.end(), b->scenes[i]) - uniq.begin());
        drd::Scene &S = b->items[i].S;
        S.nodes = b->arena_nodes;
        S.gbox = b->arena_gbox;
        S.gbox_ref = b->arena_gbox;   // batches do not run the counting traversal
        S.leaf_tris = b->arena_leaf;
        if (S.root_child >= 0) S.root_child += (int)(node_off[k] / 8);
        S.root_leaf_first += (int)leaf_off[k];
    }
    return DR_OK;
}

dr_status dr_batch_create(const dr_batch_item *items, int32_t n, dr_batch **out) try {
    if (!out) return fail(DR_E_ARG, "dr_batch_create: out is NULL");
    *out = nullptr;
    if (!items || n <= 0) return fail(DR_E_ARG, "dr_batch_create: empty batch");
    dr_batch *b = new (std::nothrow) dr_batch();
    if (!b) return fail(DR_E_NOMEM, "dr_batch_create: out of host memory");
    b->items.resize(n);
    long long path = 0;
    long long slot = 0;
    for (int i = 0; i < n; i++) {
        const dr_batch_item &it = items[i];
        dr_status st = dr_internal_make_item(it.scene, &it.camera, it.fb, it.start_block, it.end_block, &it.params, "dr_batch_create", b->items[i]);
        if (st != DR_OK) {
            delete b;
            return st;
        }
        if (i > 0 && it.params.mode != items[0].params.mode) {
            delete b;
            return fail(DR_E_ARG, "dr_batch_create: all jobs of a batch must use the same render mode");
        }
        drk::Item &I = b->items[i];
        I.slot_begin = (int)slot;
        I.path_begin = path;
        slot += I.n_slots;
        path += (long long)I.n_slots * I.spp;
        b->max_bounces = std::max(b->max_bounces, I.max_bounces);
        if (I.mode == DR_MODE_REFERENCE) b->max_lights = std::max(b->max_lights, I.S.shadow_photons);
        b->scenes.push_back(it.scene);
        b->params.push_back(it.params);
    }
    if (slot > (1LL << 30)) {
        delete b;
        return fail(DR_E_CAPACITY, "dr_batch_create: more than 2^30 pixel slots");
    }
    b->mode = items[0].params.mode;
    b->total_paths = path;
    b->total_slots = (int)slot;
    for (int i = 1; i < n; i++) {
        if (b->mode == DR_MODE_REFERENCE && b->items[i].clip != b->items[0].clip) {
            delete b;
            return fail(DR_E_ARG, "dr_batch_create: all jobs of a reference-mode batch must use the same backface culling");
        }
    }
    dr_status ast = build_arena(b);
    if (ast != DR_OK) {
        delete b;
        return ast;
    }
    cudaError_t e = upload(&b->items_dev, b->items.data(), b->items.size());
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "dr_batch_create: job table");
    }
    *out = b;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_batch_create");
}

dr_status dr_batch_set_iteration(dr_batch *b, int32_t iteration) try {
    if (!b) return fail(DR_E_ARG, "dr_batch_set_iteration: batch is NULL");
    for (size_t i = 0; i < b->items.size(); i++) {
        drk::Item &I = b->items[i];
        I.sample_base = (uint32_t)((iteration < 1 ? 0 : iteration - 1) * I.spp);
        I.blend = (iteration <= 1) ? 1.0f : (1.0f / (float)iteration);
    }
    cudaError_t e = b->done ? cudaEventSynchronize(b->done) : cudaSuccess;   // previous render finished with the table
    if (e == cudaSuccess)
        e = cudaMemcpy(b->items_dev, b->items.data(), sizeof(drk::Item) * b->items.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "dr_batch_set_iteration");
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_batch_set_iteration");
}

dr_status dr_batch_render(dr_renderer *r, dr_batch *b, int32_t use_graph, void *stream_ptr) try {
    if (!r || !b) return fail(DR_E_ARG, "dr_batch_render: NULL argument");
    if (r->counting && b->arena_node_count >= (int64_t(1) << 24))
        return fail(DR_E_CAPACITY, "dr_batch_render: traversal counting supports at most 2^24 octree nodes per batch");
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    dr_status st = ensure_accum(r, (size_t)b->total_slots);
    if (st != DR_OK) return st;
    drk::WaveDesc W;
    std::memset(&W, 0, sizeof(W));
    W.inl = b->items[0];
    W.items = b->items_dev;
    W.n_items = (int)b->items.size();
    W.mode = b->mode;
    W.max_bounces = b->max_bounces;
    W.adjoint = false;
    wave_buffers(r, W);
    const long long wave = lane_wave(b->total_paths, wave_size(r, b->mode == DR_MODE_REFERENCE ? b->max_lights : 1, 1LL << 40),
                                     r->lanes);
    if (!b->done) {
        cudaError_t e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            b->done = nullptr;
            return cuda_fail(e, "dr_batch_render: event");
        }
    }
    const int lanes = lanes_used(b->total_paths, wave, r->lanes);
    if (!use_graph) {
        st = run_waves(r, W, b->total_paths, wave, b->total_slots, stream, &r->prof, r->counting, true, lanes);
        if (st == DR_OK) cudaEventRecord(b->done, stream);
        return st;
    }
    if (b->exec == nullptr || b->graph_scratch != r->scratch_id || b->graph_wave != wave || b->graph_lanes != lanes ||
        b->graph_shape != r->shape) {
        // lane scratch is allocated before the capture (no allocation while capturing); the lanes'
        // streams join the capture through the fork event and leave it through their done events
        if (lanes > 1) {
            st = ensure_lanes(r, lanes - 1);
            if (st != DR_OK) return st;
        }
        b->drop_graph();
        cudaError_t e = cudaSuccess;
        if (!b->capture_stream) e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "dr_batch_render: capture stream");
        cudaStream_t cs = b->capture_stream;
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "dr_batch_render: begin capture");
        long long launches = r->launches;
        st = run_waves(r, W, b->total_paths, wave, b->total_slots, cs, nullptr, false, true, lanes);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cs, &g);   // always ends the capture, also after a failed launch
        r->launches = launches;
        if (st != DR_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            return st != DR_OK ? st : cuda_fail(e, "dr_batch_render: end capture");
        }
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            b->exec = nullptr;
            return cuda_fail(e, "dr_batch_render: instantiate");
        }
        b->graph = g;
        b->graph_scratch = r->scratch_id;
        b->graph_wave = wave;
        b->graph_lanes = lanes;
        b->graph_shape = r->shape;
        size_t nodes = 0;
        cudaGraphGetNodes(g, nullptr, &nodes);
        b->graph_launches = 0;
        // kernel nodes only (the accumulator clear is a memset node)
        std::vector<cudaGraphNode_t> list(nodes);
        if (nodes && cudaGraphGetNodes(g, list.data(), &nodes) == cudaSuccess) {
            for (size_t k = 0; k < nodes; k++) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(list[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) b->graph_launches++;
            }
        }
    }
    cudaError_t e = cudaGraphLaunch(b->exec, stream);
    if (e != cudaSuccess) return cuda_fail(e, "dr_batch_render: graph launch");
    cudaEventRecord(b->done, stream);
    r->launches += b->graph_launches;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_batch_render");
}

int64_t dr_batch_paths(const dr_batch *b) { return b ? b->total_paths : 0; }

void dr_batch_destroy(dr_batch *b) { delete b; }

}  // extern "C"

const drd::Scene *dr_internal_scene_device(const dr_scene *scene) { return scene ? &scene->dev : nullptr; }

bool dr_internal_scene_textures_ok(const dr_scene *scene) { return scene && scene->max_texture <= scene->n_textures; }

void dr_internal_set_error(const char *msg) { g_err = msg ? msg : ""; }

dr_status dr_internal_exception(const char *where) noexcept {
    const char *what = "unexpected exception";
    dr_status s = DR_E_STATE;
    try {
        throw;
    } catch (const std::bad_alloc &) {
        what = "out of host memory";
        s = DR_E_NOMEM;
    } catch (const std::exception &e) {
        what = e.what();
    } catch (...) {
    }
    try {
        g_err = std::string(where) + ": " + what;
    } catch (...) {  // no memory left even for the message: keep the status
    }
    return s;
}
