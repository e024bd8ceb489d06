/*
 * dr_api.h - C ABI of the GB300-native DumbRay rendering hot path.
 *
 * Drop-in boundary: this library replaces the per-pixel path tracer that DumbRay plugs under its
 * block renderer, i.e. the pair of virtuals
 *     BlockRenderer::renderBlocksCPU / renderBlocksGPU
 *       (__source__/DataStructures/Renderers/BlockRenderer/BlockRenderer.cuh:43-44)
 * implemented by DumbRenderer (__source__/DataStructures/Renderers/DumbRenderer/DumbRenderer.cu:52-113),
 * together with the function packs that path calls: Octree cast, Shader, Lense, Light and the
 * block-based frame buffer.  Every entry point is extern "C", takes plain pointers and sizes, and
 * returns a dr_status; there is no CPU fallback.  No C++ exception leaves the library: a host
 * allocation failure inside a call returns DR_E_NOMEM, any other exception DR_E_STATE.  Device pointers are CUDA device memory owned by
 * the caller unless stated otherwise; `stream` is a cudaStream_t passed as void*.
 *
 * Threading: a dr_scene is immutable after creation and may be shared by any number of threads.
 * A dr_renderer owns per-caller scratch (wavefront queues) and must be used by one thread / one
 * stream at a time, mirroring the reference's one DeviceBlockManager per GPU worker thread
 * (__source__/DataStructures/Screen/FrameBuffer/FrameBuffer.impl.cuh:271-317).
 */
#ifndef DR_API_H
#define DR_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t dr_status;
#define DR_OK 0
#define DR_E_ARG 1       /* invalid argument (null pointer, bad size, bad enum) */
#define DR_E_CUDA 2      /* a CUDA runtime call failed; see dr_last_error() */
#define DR_E_CAPACITY 3  /* a caller-provided capacity is too small */
#define DR_E_TIMEOUT 4   /* a bounded device-side wait gave up */
#define DR_E_NOMEM 5     /* host or device allocation failed */
#define DR_E_STATE 6     /* object used in a state that does not allow the call */

typedef struct dr_scene dr_scene;
typedef struct dr_renderer dr_renderer;

/* ---- octree build parameters -------------------------------------------------------------
 * Octree.cuh:10-13: OCTREE_MAX_DEPTH 24, OCTREE_POLYCOUNT_TO_SPLIT_NODE 8; Octree.impl.cuh:3-5:
 * OCTREE_AABB_EPSILON 1.28e-3 (box_epsilon, the padding of octant and leaf boxes).  Zero fields
 * take those defaults; threads = 0 uses every host core.  The reference's values reproduce its
 * tree exactly (casts and per-ray box / triangle test counts).  The closest hit itself does not
 * depend on the tree up to exact ties, so a scene rendered only in the physical mode may take a
 * box_epsilon scaled to its coordinates (an absolute 1.28e-3 is a large fraction of the leaf cells
 * of a finely tessellated unit-size mesh, which duplicates triangles into many leaves):
 * box_epsilon > 0 is used as given, box_epsilon < 0 selects 2^-18 x the largest absolute vertex
 * coordinate (margin for the rounding of hit points in the leaf-box acceptance test).  Traversals
 * skip octree boxes lying entirely behind the ray origin, which the reference's slab test keeps
 * (clipBackface = false) although no hit at t > 0 can come of them; dr_cast_counted, whose counts
 * reproduce the reference's, keeps them on scenes built with box_epsilon = 0.
 * split_threshold: 0 = the reference's 8.  With a scene-scaled box_epsilon smaller leaves pay: a
 * 1.31M-triangle displaced sphere path-traces fastest at 3-4 (793 Mpaths/s against 754 at 8). */
typedef struct {
    int32_t max_depth;
    int32_t split_threshold;
    int32_t threads;
    float box_epsilon;
    /* 1: build on the current CUDA device (per-reference clipping and per-node passes on the GPU,
     * level bookkeeping on the host); the tree is bit-identical to the host build.  0: host threads. */
    int32_t device_build;
} dr_build_params;

/* ---- materials --------------------------------------------------------------------------
 * Reference-semantics shaders (Material<BakedTriFace> function packs):
 *   DR_MAT_DUMB_BASED        DumbBasedShader(fresnel, specular, diffuse=color, metal)
 *                            (__source__/.../Shaders/DumbBasedShader/DumbBasedShader.impl.cuh:5-122)
 *   DR_MAT_SIMPLE_STOCHASTIC SimpleStochasticShader(albedo=color, diffuse, smoothness, shininess)
 *                            (__source__/.../Shaders/SimpleStochasticShader/SimpleStochasticShader.impl.cuh:4-37)
 *   DR_MAT_FRESNEL           Shaders::FresnelShader(fresnel=color): no indirect samples, Schlick term
 *                            of the interpolated normal (.../Shaders/FresnelShader/FresnelShader.impl.cuh:5-19)
 *   DR_MAT_DEFAULT           DefaultShaderGeneric(albedo=color, diffuse, smoothness, shininess): one
 *                            mirror-direction sample, diffuse + Phong lobe (.../Shaders/DefaultShader/
 *                            DefaultShader.impl.cuh:3-52)
 * Physical-mode materials (no reference counterpart; albedo = color, overridable per triangle):
 *   DR_MAT_LAMBERT, DR_MAT_MIRROR, DR_MAT_GLOSSY (GGX, alpha = roughness).  In the physical mode the
 *   reference-semantics types shade as Lambert with their colour. */
#define DR_MAT_DUMB_BASED 0
#define DR_MAT_SIMPLE_STOCHASTIC 1
#define DR_MAT_LAMBERT 2
#define DR_MAT_MIRROR 3
#define DR_MAT_GLOSSY 4
#define DR_MAT_FRESNEL 5
#define DR_MAT_DEFAULT 6

/* Reference-mode textures (ColoredTexture, __source__/.../Components/DumbStructs.cuh:70-131): a
 * textured channel is its colour x the texel at (uv x tiling + offset), uv interpolated from the
 * triangle's corner coordinates (dr_scene_set_textures).  texture[k] is a 1-based index into the
 * scene's textures, 0 = none (so zero-initialised materials are untextured).  Channels:
 *   DR_TEX_COLOR   DUMB_BASED diffuse, FRESNEL colour
 *   DR_TEX_FRESNEL DUMB_BASED fresnel
 *   DR_TEX_NORMAL  DUMB_BASED normal map (tangent frame from the corner uv; normal_color weights it)
 *   DR_TEX_ALPHA   DUMB_BASED alpha cutout: where the texel's alpha <= alpha_threshold the surface
 *                  passes paths and photons straight through */
#define DR_TEX_COLOR 0
#define DR_TEX_FRESNEL 1
#define DR_TEX_NORMAL 2
#define DR_TEX_ALPHA 3

typedef struct {
    int32_t type;
    float color[3];
    float fresnel[3];
    float specular;
    float metal;
    float diffuse;
    float smoothness;
    float shininess;
    float roughness;
    float emission[3];
    int32_t texture[4];
    float tiling[4][2];
    float offset[4][2];
    float normal_color[3];
    float alpha_threshold;
} dr_material;

/* ---- lights (reference semantics; Light function pack, Light.cuh:14-59) -----------------
 *   DR_LIGHT_SPHERICAL         SphericalLightEmitter(color, position, radius)
 *   DR_LIGHT_SOFT_DIRECTIONAL  SimpleSoftDirectionalLight(color, direction, distance, softness)
 *   DR_LIGHT_DIRECTIONAL       SimpleDirectionalLight(color, direction, distance)
 *   DR_LIGHT_SPOTLIGHT         Lights::Spotlight(color, luminosity, position, direction, hotspot_angle,
 *                              falloff_angle, falloff_power, emitter_size, emit_from_sphere, cast_shadows,
 *                              samples) (.../Scene/Lights/Spotlight/Spotlight.impl.cuh:5-79): `samples`
 *                              photons per shading point (0..16) from a disc or sphere emitter with a
 *                              cone falloff; cast_shadows = 0 lights without an occlusion test.
 * At most 16 lights per scene. */
#define DR_LIGHT_SPHERICAL 0
#define DR_LIGHT_SOFT_DIRECTIONAL 1
#define DR_LIGHT_DIRECTIONAL 2
#define DR_LIGHT_SPOTLIGHT 3

typedef struct {
    int32_t type;
    float color[3];
    float position[3];
    float direction[3];
    float radius;
    float distance;
    float softness;
    /* DR_LIGHT_SPOTLIGHT only (angles in degrees) */
    float luminosity;
    float hotspot_angle;
    float falloff_angle;
    float falloff_power;
    float emitter_size;
    int32_t emit_from_sphere;
    int32_t cast_shadows;
    int32_t samples;
} dr_light;

/* ---- camera / lenses (Lense function pack, Lense.cuh:46-82; Camera.impl.cuh:7-14) --------
 *   DR_LENS_DEFAULT_PERSPECTIVE  DefaultPerspectiveLense(angle[0])   (normalised pinhole)
 *   DR_LENS_SIMPLE_STOCHASTIC    SimpleStochasticLense(angle[0])     (jittered, unnormalised)
 *   DR_LENS_SPHERICAL_SEGMENT    Lenses::SphericalSegmentLense(angle, focal_distance, softness, filter)
 * Physical mode only:
 *   DR_LENS_PINHOLE   jittered pinhole, vertical fov angle[0]
 *   DR_LENS_FISHEYE   equidistant fisheye, angle[0] = full field of view across the image height
 *   DR_LENS_SPHERICAL latitude/longitude, angle[0] x angle[1] degrees per unit screen space
 * Camera space is +x right, +y up, +z forward; world direction = x*right + y*up + z*forward,
 * origin = position + (lens origin expressed in the same basis).
 * origin_rows = 1 maps lens origins the way the reference's Camera does (Camera.impl.cuh:7-10,
 * `ray >>= transform`; Transform.impl.h:84-90): o -> (o.row_x, o.row_y, o.row_z) + position, while
 * directions keep the right / up / forward combination (Transform::direction, Transform.impl.h:166).
 * The two differ for a rotated camera (the rows are the transpose of the direction basis, times the
 * scale); only the spherical-segment lens has origins off the camera position.  Zero-initialised
 * cameras keep the basis mapping.
 * lens_x > 0: the focal factor of DR_LENS_DEFAULT_PERSPECTIVE / DR_LENS_SIMPLE_STOCHASTIC used as
 * given (the `x` a reference lens stores, DefaultPerspectiveLense.impl.cuh:5-9,
 * SimpleStochasticLense.impl.cuh:4-9), so a host that holds constructed reference lenses passes
 * them on exactly; 0 (zero-initialised): 0.5 / tan(angle[0] / 2), angle clamped to [1, 179]
 * degrees, as the lens constructors compute it. */
#define DR_LENS_DEFAULT_PERSPECTIVE 0
#define DR_LENS_SIMPLE_STOCHASTIC 1
#define DR_LENS_SPHERICAL_SEGMENT 2
#define DR_LENS_PINHOLE 3
#define DR_LENS_FISHEYE 4
#define DR_LENS_SPHERICAL 5

typedef struct {
    int32_t lens;
    float angle[2];
    float focal_distance;
    float softness;
    float filter[3];
    float position[3];
    float right[3];
    float up[3];
    float forward[3];
    int32_t origin_rows;
    float row_x[3];
    float row_y[3];
    float row_z[3];
    float lens_x;
} dr_camera;

/* ---- render parameters ---------------------------------------------------------------------
 * DR_MODE_REFERENCE: DumbRenderer's estimator (DumbRenderer.cu:174-443): fsaa samples_x x
 *   samples_y sub-pixels, max_bounces indirect layers, analytic-light NEE cast from the light
 *   toward the point, backface culling flag, HEIGHT/WIDTH/MIN/MAX boxing (DumbRenderer.cu:190-200).
 * DR_MODE_PHYSICAL: unbiased path tracer over emissive triangles with Lambert/mirror/GGX,
 *   samples_x*samples_y jittered samples per pixel, max_bounces = path depth.
 * iteration: 1-based progressive index; blend = (iteration <= 1) ? 1 : 1/iteration
 *   (DumbRenderer.cu:64,102).  Random numbers are counter-based, keyed by
 *   (seed, pixel, sample, bounce, dimension), so any sample is reproducible. */
#define DR_MODE_REFERENCE 0
#define DR_MODE_PHYSICAL 1

#define DR_BOXING_HEIGHT 0
#define DR_BOXING_WIDTH 1
#define DR_BOXING_MIN 2
#define DR_BOXING_MAX 3

typedef struct {
    int32_t mode;
    int32_t width;
    int32_t height;
    int32_t samples_x;
    int32_t samples_y;
    int32_t max_bounces;
    int32_t cull_backfaces;
    int32_t boxing;
    int32_t iteration;
    uint32_t seed;
} dr_render_params;

/* Frame buffer: BlockBasedFrameBuffer<8,16> layout (BlockBasedFrameBuffer.cuh:91,
 * BlockBasedFrameBuffer.impl.cuh:108-156): float4 data[128*blockId + pixelId],
 * blockId = by*ceil(W/8) + bx, pixelId = oy*8 + ox. */
#define DR_BLOCK_W 8
#define DR_BLOCK_H 16

/* ---- library ------------------------------------------------------------------------------ */

/* Message of the last failing call on this thread (never NULL). */
const char *dr_last_error(void);

/* Library / ABI version (major*10000 + minor*100 + patch). */
int32_t dr_version(void);

/* ---- host octree (no device work) ----------------------------------------------------------
 * The octree alone, built on the host with the reference's split rule (Octree.impl.cuh:97-129,
 * 339-533) and kept in host memory, e.g. to inspect or cache it.  Export layout is the same as
 * dr_scene_export_tree (node 0 = root). */
typedef struct dr_octree dr_octree;
dr_status dr_octree_create_host(const float *xyz, int32_t n, const dr_build_params *bp, dr_octree **out);
dr_status dr_octree_stats(const dr_octree *tree, int64_t *nodes, int64_t *leaves, int64_t *refs, int32_t *depth);
dr_status dr_octree_export(const dr_octree *tree, float *node_box, int32_t *node_child, int32_t *node_leaf, int32_t *leaf_tri);
/* The group-test boxes the traversal reads for this tree (no reference counterpart; they replace the
 * child-box reads of Octree::cast, Octree.impl.cuh:174-212, without changing any hit or count):
 * float[(nodes - 1) / 8][48] each; group g (the 8 children of an inner node: export nodes 8g + 1 ..
 * 8g + 8) holds planes lo x, lo y, lo z, hi x, hi y, hi z of its 8 children.  gbox: boxes refitted to the non-empty
 * leaves below each child (a leaf's own box; an inner child's union of its non-empty children's
 * refitted boxes); gbox_ref: the reference's boxes.  In both an empty leaf (and in gbox a subtree
 * without triangles) is the point (1e30, 1e30, 1e30).  Either pointer may be NULL. */
dr_status dr_octree_group_planes(const dr_octree *tree, float *gbox, float *gbox_ref);
void dr_octree_destroy(dr_octree *tree);

/* ---- scene ---------------------------------------------------------------------------------
 * Replaces Octree<Renderable<BakedTriFace>>::push + build (Octree.impl.cuh:97-129) and the lazy
 * device upload of the scene (ReferenceManager::gpuHandle, ReferenceManager.impl.cuh:18-51).
 * xyz: host float[n][3][3] triangle vertices; nrm: host float[n][3][3] per-vertex normals or NULL
 * (flat shading); mat_id: host int32[n] or NULL (all 0).  The octree is built on the host with the
 * reference's split rule and uploaded once; triangle index i is the push order. */
dr_status dr_scene_create(const float *xyz, const float *nrm, const int32_t *mat_id, int32_t n,
                          const dr_material *mats, int32_t n_mats, const dr_light *lights, int32_t n_lights,
                          const dr_build_params *bp, dr_scene **out);

/* Physical-mode per-triangle overrides (host arrays, any may be NULL): albedo float[n][3],
 * emission float[n][3], roughness float[n]. */
dr_status dr_scene_set_triangle_params(dr_scene *scene, const float *albedo, const float *emission,
                                       const float *roughness);

/* Texture images (Texture, __source__/.../Components/Texture/Texture.impl.cuh:81-95): host RGBA
 * float[height][width][4], row 0 = the image's first row (texture[y][x]); lookups wrap u and v into
 * [0, 1), flip v and take the nearest texel (DR_FILTER_NONE) or blend four (DR_FILTER_BILINEAR), as
 * the reference does. */
#define DR_FILTER_NONE 0
#define DR_FILTER_BILINEAR 1
typedef struct {
    int32_t width;
    int32_t height;
    int32_t filtering;
    const float *rgba;
} dr_texture;

/* Sets the scene's textures (copied to the device; replaces earlier ones) and per-corner texture
 * coordinates uv: host float[n][3][2] (BakedTriFace::tex x / y), or NULL for all zeros.  Every
 * material texture index must be <= n_textures; renders of a scene whose materials use textures
 * fail until they are set.  Batches created before a later call keep the earlier textures, so their
 * device memory is released with the scene (dr_scene_destroy), not by the next call. */
dr_status dr_scene_set_textures(dr_scene *scene, const dr_texture *textures, int32_t n_textures, const float *uv);

/* Device pointers to the scene's per-triangle albedo and emission (float[n][3] each), for
 * callers that update them in place (e.g. an optimiser).  Emissive-triangle sampling tables are
 * not rebuilt by in-place writes; call dr_scene_set_triangle_params to change which are emissive. */
dr_status dr_scene_triangle_params_device(dr_scene *scene, float **albedo, float **emission);

/* Octree statistics: node count, leaf count, total leaf references, tree depth. */
dr_status dr_scene_stats(const dr_scene *scene, int64_t *nodes, int64_t *leaves, int64_t *refs, int32_t *depth);

/* Copies the flattened octree to host arrays for inspection (sizes from dr_scene_stats):
 * node_box float[nodes][6] (min xyz, max xyz), node_child int32[nodes] (first child or -1),
 * node_leaf int32[nodes][2] (first ref, ref count; zeros for inner nodes), leaf_tri int32[refs]. */
dr_status dr_scene_export_tree(const dr_scene *scene, float *node_box, int32_t *node_child,
                               int32_t *node_leaf, int32_t *leaf_tri);

void dr_scene_destroy(dr_scene *scene);

/* ---- ray casting ---------------------------------------------------------------------------
 * Replaces Octree<...>::cast (Octree.impl.cuh:174-212) / Raycaster::cast (Raycaster.cuh:75-83):
 * closest hit in units of |direction| (directions are not normalised), backface culling flag,
 * self-hit avoidance by object identity (validateNotSameAsObject, Octree.impl.cuh:126):
 * ignore_tri int32[n] or NULL (-1 = none).
 * Device arrays: origin float[n][3], direction float[n][3]; outputs hit_tri int32[n] (-1 = miss),
 * hit_t float[n] (FLT_MAX on a miss). */
dr_status dr_cast(const dr_scene *scene, const float *origin, const float *direction, const int32_t *ignore_tri,
                  int32_t n, int32_t cull_backfaces, int32_t *hit_tri, float *hit_t, void *stream);

/* Same as dr_cast, also writing per-ray traversal counters (device int32[n] each): child-box slab
 * tests and triangle tests.  Used to compute the algorithmic bytes per ray. */
dr_status dr_cast_counted(const dr_scene *scene, const float *origin, const float *direction, const int32_t *ignore_tri,
                          int32_t n, int32_t cull_backfaces, int32_t *hit_tri, float *hit_t,
                          int32_t *box_tests, int32_t *tri_tests, void *stream);

/* ---- block renderer ------------------------------------------------------------------------
 * A renderer owns the wavefront scratch (ray / hit / shadow queues, per-pixel accumulators) for
 * at most `wave_paths` paths in flight (0 = default 4Mi, about 1.2 GB of scratch per lane).  Large
 * renders run faster with larger waves (fewer per-wave launch sequences): a 1920x1080 x 64 spp
 * physical-mode frame renders about 4.5% faster with 16Mi (about 5 GB per lane). */
dr_status dr_renderer_create(int32_t wave_paths, dr_renderer **out);
void dr_renderer_destroy(dr_renderer *r);

/* Concurrent wave pipelines ("lanes") of one dr_render_blocks call, 1..DR_MAX_LANES (default
 * DR_DEFAULT_LANES): the waves of a render alternate over `lanes` scratch sets, each on its own
 * stream forked from and joined back into the caller's stream, adding into one accumulator, so one
 * pipeline's kernels fill the tails of another's (the reference runs several GPU worker threads
 * per device for the same reason, Renderer::ThreadConfiguration).  Each extra lane allocates a
 * scratch set like the renderer's own on first use.  Results do not depend on the lane count
 * beyond float accumulation order.  Batches and the adjoint use one lane. */
#define DR_DEFAULT_LANES 4
#define DR_MAX_LANES 8
dr_status dr_renderer_set_lanes(dr_renderer *r, int32_t lanes);
int32_t dr_renderer_lanes(const dr_renderer *r);

/* Block shape of the traversal kernels (no counterpart in the reference, which launches one
 * thread per pixel): 0 = 256 threads x 3 blocks per SM (default), 1 = 128 threads x 6 blocks per SM.
 * Both cap registers at 80 and keep the same threads in flight; they differ in how warps share an
 * SM's blocks and leave the tail of a launch.  Results do not depend on the shape.  A batch graph
 * captured with one shape is re-captured when the renderer's shape changes. */
dr_status dr_renderer_set_block_shape(dr_renderer *r, int32_t shape);
int32_t dr_renderer_block_shape(const dr_renderer *r);

/* Replaces DumbRenderer::renderBlocksGPU (DumbRenderer.cu:87-113): renders blocks
 * [start_block, end_block) of a width x height image into the caller's device frame buffer
 * (BlockBasedFrameBuffer<8,16> layout, float4), setting (iteration <= 1) or blending (1/iteration)
 * each pixel exactly like setBlockPixelColor / blendBlockPixelColor.  Asynchronous on `stream`. */
dr_status dr_render_blocks(dr_renderer *r, const dr_scene *scene, const dr_camera *camera, float *fb_blockmajor,
                           int32_t start_block, int32_t end_block, const dr_render_params *params, void *stream);

/* ---- differentiable rendering (no reference counterpart) -------------------------------------
 * Path-replay adjoint of the physical-mode render: given dL/dI for the pixels of blocks
 * [start_block, end_block) (block-major float4, device), ADDS dL/d albedo and dL/d emission
 * (device float[n][3] each) for the scene's triangles.  The paths are regenerated from the
 * counter-based random numbers of `params` (same seed / iteration as the forward render), so no
 * path is stored between the passes: memory is the renderer's wave scratch plus one triangle id
 * per path vertex of the paths in flight.  Sampling pdfs (light selection, BSDF, MIS) are treated
 * as constants, which keeps the gradient estimate unbiased. */
dr_status dr_render_adjoint(dr_renderer *r, const dr_scene *scene, const dr_camera *camera, const float *dl_dfb_blockmajor,
                            int32_t start_block, int32_t end_block, const dr_render_params *params, float *grad_albedo,
                            float *grad_emission, void *stream);

/* ---- batches (no reference counterpart) -------------------------------------------------------
 * Many independent render jobs (scenes, cameras, frame buffers, resolutions, sample counts) whose
 * paths share the same wavefront waves, so small jobs fill the GPU together.  All jobs of a batch
 * use the same render mode.  dr_batch_render with use_graph = 1 captures the whole launch
 * sequence once into a CUDA graph (per renderer scratch set, captured on a private stream, so the
 * caller's stream may be the legacy default stream) and replays it on the caller's stream;
 * dr_batch_set_iteration changes the progressive iteration of every job without re-capturing (it
 * first waits for the batch's previous render, which reads the same job table).  A batch must not
 * be rendered on two streams at once, and a renderer's scratch serves one render at a time. */
typedef struct dr_batch dr_batch;
typedef struct {
    const dr_scene *scene;
    dr_camera camera;
    dr_render_params params;
    float *fb;
    int32_t start_block, end_block;
} dr_batch_item;

dr_status dr_batch_create(const dr_batch_item *items, int32_t n, dr_batch **out);
dr_status dr_batch_set_iteration(dr_batch *batch, int32_t iteration);
dr_status dr_batch_render(dr_renderer *r, dr_batch *batch, int32_t use_graph, void *stream);
int64_t dr_batch_paths(const dr_batch *batch);
void dr_batch_destroy(dr_batch *batch);

/* Allocation-free variant of dr_render_blocks.  It has no counterpart in the reference: it exists
 * for callers that cannot allocate device memory while they render (a plugin host whose device
 * memory belongs to another allocator's pool or fixed budget, a latency-critical render thread that
 * must not let cudaMalloc/cudaFree synchronise the device).  Same arguments, results
 * and blending as dr_render_blocks, but no dr_renderer: the scratch is one file-scope device array
 * of DR_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until process exit.
 * At most DR_NOALLOC_MAX_BLOCKS blocks per call (more returns DR_E_CAPACITY).  All calls share the
 * array: calls whose work overlaps on the GPU race, so issue them on one stream.  The first call on
 * a device looks up the array's address with that device current; make it before any stream
 * capture starts.  Calls no cudaMalloc, cudaFree or allocating library routine. */
#define DR_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
#define DR_NOALLOC_MAX_BLOCKS 2048
dr_status dr_render_blocks_noalloc(const dr_scene *scene, const dr_camera *camera, float *fb_blockmajor,
                                   int32_t start_block, int32_t end_block, const dr_render_params *params, void *stream);

/* Number of blocks of a width x height image (ceil(W/8) * ceil(H/16)). */
int32_t dr_block_count(int32_t width, int32_t height);

/* Kernel launches issued by this renderer since creation (for launch accounting). */
int64_t dr_renderer_launch_count(const dr_renderer *r);

/* ---- instrumentation ---------------------------------------------------------------------
 * Kernel classes timed with CUDA events recorded on the launch stream around each launch. */
#define DR_KERNEL_CAMERA 0
#define DR_KERNEL_TRACE 1
#define DR_KERNEL_SHADE 2
#define DR_KERNEL_SHADOW 3
#define DR_KERNEL_RESOLVE 4
#define DR_KERNEL_CLASSES 5

/* Enables (1) or disables (0) per-class event timing for subsequent dr_render_blocks calls and
 * clears the accumulated times. */
dr_status dr_renderer_set_profiling(dr_renderer *r, int32_t enable);

/* Waits for the recorded events and returns, per kernel class, the summed launch durations in
 * milliseconds and the number of timed launches (arrays of DR_KERNEL_CLASSES; either may be NULL). */
dr_status dr_renderer_kernel_times(dr_renderer *r, double *ms, int64_t *launches);

/* Per kernel class, the busy time in milliseconds since profiling was enabled: the length of the
 * union of the class's launch intervals over all lanes (equal to the summed durations with one
 * lane; less when launches of several lanes overlap).  busy_ms[DR_KERNEL_CLASSES]. */
dr_status dr_renderer_kernel_busy(dr_renderer *r, double *busy_ms);

/* Counting pass: while enabled, trace and shadow kernels also count, per cast, the reference's
 * child-box slab tests and triangle tests (see dr_cast_counted).  Slower; never on a timed path. */
dr_status dr_renderer_set_counting(dr_renderer *r, int32_t enable);

/* Accumulated counts since counting was enabled (synchronises the device): counts[6] =
 * {extension rays, their box tests, their triangle tests, shadow casts, their box tests, their triangle tests}. */
dr_status dr_renderer_counters(dr_renderer *r, int64_t *counts);

/* Queue sizes of the last wave the renderer ran on its own scratch (its first lane), per bounce b < n
 * (n <= 68; synchronises the device): rays[b] extension rays traced at bounce b (b = 0: camera rays),
 * shadow_records[b] shadow rays (physical mode) or light photons (reference mode) queued at bounce b.
 * With one lane and a wave at least as large as a render, these are the render's own counts - path
 * survival per bounce, and the rays of each trace launch for profiling.  No reference counterpart. */
dr_status dr_renderer_wave_counts(dr_renderer *r, int32_t *rays, int32_t *shadow_records, int32_t n);

/* ---- images (host memory) ----------------------------------------------------------------
 * Replace Images::saveBufferPNG (__source__/Namespaces/Images/Images.cu:22-40) and the frame
 * buffer's getColor walk it does.  rgba is a row-major float[height][width][4] image. */

/* Block-major frame buffer (DR_BLOCK_W x DR_BLOCK_H blocks, host copy) -> row-major rgba. */
dr_status dr_image_from_blocks(const float *fb_blockmajor, int32_t width, int32_t height, float *rgba);

/* The reference's 8-bit conversion of every channel: v = 255*c; v > 255 -> 255, v < 0 -> 0, else
 * truncated (Images.cu:7-12).  out: uint8[height][width][4]. */
dr_status dr_image_to_rgba8(const float *rgba, int32_t width, int32_t height, uint8_t *out);

/* 8-bit RGBA PNG of those bytes (stored-deflate zlib stream; any PNG reader decodes the same
 * pixels as the reference's lodepng file). */
dr_status dr_image_write_png(const float *rgba, int32_t width, int32_t height, const char *path);

/* Portable float map (RGB, little-endian, rows bottom-up): the unclamped radiance. */
dr_status dr_image_write_pfm(const float *rgba, int32_t width, int32_t height, const char *path);

/* PNG decoding for textures (Images::getTexturePNG, Images.cu:38-56, which takes lodepng's 8-bit RGBA
 * output): every colour type and bit depth, tRNS, Adam7.  Writes width / height and, when rgba8 is
 * not NULL, uint8[height][width][4] (row 0 = the file's first row); call with rgba8 = NULL first for
 * the size.  Texture texels are these bytes / 255. */
dr_status dr_png_read(const char *path, int32_t *width, int32_t *height, uint8_t *rgba8);

/* ---- OBJ meshes (host) -----------------------------------------------------------------------
 * Replace MeshReader::readObj + PolyMesh::bake (__source__/Namespaces/MeshReader/MeshReader.impl.h:
 * 160-367, __source__/DataStructures/Objects/Meshes/PolyMesh/PolyMesh.impl.h:140-152) with the same
 * reading rules: objects are the face ranges between `g` lines, x of vertices and normals is mirrored,
 * missing normals come from generated vertex normals, polygons become triangle fans.  Each object's
 * triangles are float[n][3][3] (xyz), with per-corner normals and texture coordinates of the same
 * shape, ready for dr_scene_create. */
typedef struct dr_mesh_file dr_mesh_file;
dr_status dr_obj_read(const char *path, dr_mesh_file **out);
int32_t dr_mesh_file_objects(const dr_mesh_file *m);
const char *dr_mesh_file_object_name(const dr_mesh_file *m, int32_t object);
int32_t dr_mesh_file_object_triangles(const dr_mesh_file *m, int32_t object);
/* Any of xyz / nrm / uv may be NULL. */
dr_status dr_mesh_file_object_data(const dr_mesh_file *m, int32_t object, float *xyz, float *nrm, float *uv);
void dr_mesh_file_destroy(dr_mesh_file *m);

/* ---- scene files (.dumb) ---------------------------------------------------------------------
 * Replace DumbRenderContext::fromFile (__source__/DataStructures/DumbRenderContext/DumbRenderContext.cu:
 * 300-372) and what it calls: the Dson text format (Namespaces/Dson/Dson.cu:225-447), "include",
 * "materials" (dumb_based with its presets, simple_stochastic, fresnel_color), "lights"
 * (simple_soft_directional, simple_spherical, spotlight), "groups" and "objects" (OBJ meshes placed by Transforms, groups with fallback /
 * override materials), "camera" (simple_stochastic / spherical_segment lenses, Transform with
 * position / rotation / scale / relative_position) and "renderer" (boxing, bounces, samples per
 * pixel, backface culling; the thread / block settings are validated and not used).  Relative paths
 * resolve against the directory of the file that names them, then the working directory.
 * Materials: dumb_based, simple_stochastic, fresnel_color; lights: simple_soft_directional,
 * simple_spherical, spotlight (everything the reference's registry holds); textures from PNG files
 * (by path or name, nearest or bilinear).  Mesh primitives (left unimplemented by the reference)
 * fail the load with a message.  The triangles come out in the reference's push order (an object that
 * names no OBJ object takes every object of the file, in file order; the reference's order there
 * is that of a hash map). */
typedef struct dr_scene_file dr_scene_file;
dr_status dr_scene_file_load(const char *path, dr_scene_file **out);
/* counts: [0] triangles, [1] materials, [2] lights. */
dr_status dr_scene_file_counts(const dr_scene_file *f, int32_t *counts);
/* Triangles (float[n][3][3]), per-corner normals (same shape) and material ids (int32[n]); any may
 * be NULL. */
dr_status dr_scene_file_geometry(const dr_scene_file *f, float *xyz, float *nrm, int32_t *mat_id);
dr_status dr_scene_file_materials(const dr_scene_file *f, dr_material *mats);
dr_status dr_scene_file_lights(const dr_scene_file *f, dr_light *lights);
/* The file's camera (origin_rows = 1) and reference-mode render parameters (width / height are 0;
 * iteration 1, seed 0). */
dr_status dr_scene_file_camera(const dr_scene_file *f, dr_camera *camera);
dr_status dr_scene_file_render_params(const dr_scene_file *f, dr_render_params *params);
/* The file's textures (PNG files its materials name; ids in dr_material.texture are 1-based into
 * this list): count, then size / filtering / texels (float[height][width][4], bytes / 255) of each. */
int32_t dr_scene_file_textures(const dr_scene_file *f);
dr_status dr_scene_file_texture(const dr_scene_file *f, int32_t i, int32_t *width, int32_t *height, int32_t *filtering,
                                float *rgba);
/* Per-corner texture coordinates of the triangles, float[n][3][2] (from the OBJ files). */
dr_status dr_scene_file_texcoords(const dr_scene_file *f, float *uv);
/* dr_scene_create over the file's geometry, materials and lights, then dr_scene_set_textures with
 * its textures and texture coordinates (DumbRenderContext::buildFromFile). */
dr_status dr_scene_file_create_scene(const dr_scene_file *f, const dr_build_params *bp, dr_scene **out);
void dr_scene_file_destroy(dr_scene_file *f);

/* ---- progressive render process -----------------------------------------------------------
 * Replaces BufferedRenderProcess (__source__/DataStructures/Renderers/BufferedRenderProcess/
 * BufferedRenderProcess.cu:42-229) without its window: a host worker thread renders iteration after
 * iteration of one view (its own dr_renderer and CUDA stream, on the device current at creation)
 * and publishes each finished image as a host row-major float4 copy.  double_buffered = 0: iterations
 * accumulate with the progressive blend until `target` iterations; 1: like the reference's double
 * buffering (swap and reset after each iteration), every frame is one fresh iteration (seed +
 * frame index) rendered while the previous frame stays readable; `target` then counts frames.
 * Changing the view restarts the count (the reference restarts on a resolution change).  Callbacks
 * run on the worker thread. */
typedef struct dr_progressive dr_progressive;
typedef void (*dr_progress_callback)(void *arg);

dr_status dr_progressive_create(const dr_scene *scene, const dr_camera *camera, const dr_render_params *params,
                                int32_t double_buffered, dr_progressive **out);
/* Iterations (frames when double-buffered) to render before idling; < 0 = until stopped (default). */
dr_status dr_progressive_set_target(dr_progressive *p, int32_t iterations);
/* New camera and/or parameters (either may be NULL); restarts the accumulation. */
dr_status dr_progressive_set_view(dr_progressive *p, const dr_camera *camera, const dr_render_params *params);
/* setIterationCompletionCallback / setRenderCompletionCallback / setErrorOnIteration. */
dr_status dr_progressive_set_callbacks(dr_progressive *p, dr_progress_callback on_iteration,
                                       dr_progress_callback on_complete, dr_progress_callback on_error, void *arg);
dr_status dr_progressive_start(dr_progressive *p);
/* Stops the worker after the iteration in flight. */
dr_status dr_progressive_stop(dr_progressive *p);
/* Waits until at least `count` iterations (frames) of the current view are complete; DR_E_TIMEOUT otherwise. */
dr_status dr_progressive_wait(dr_progressive *p, int32_t count, int32_t timeout_ms);
int32_t dr_progressive_completed(dr_progressive *p);
/* Copies the last complete image (rgba float[height][width][4]) and its iteration index. */
dr_status dr_progressive_read(dr_progressive *p, float *rgba, int32_t width, int32_t height, int32_t *iteration);
dr_status dr_progressive_save_png(dr_progressive *p, const char *path);
/* Summed wall time of the completed iterations (renderTime, BufferedRenderProcess.cu:109-115). */
double dr_progressive_render_seconds(dr_progressive *p);
void dr_progressive_destroy(dr_progressive *p);

#ifdef __cplusplus
}
#endif

#endif /* DR_API_H */
