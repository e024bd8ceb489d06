// Thin C-ABI driver around the UNMODIFIED reference DumbRay host path, compiled together with the
// reference's own sources by oracle/build_ref.sh into oracle/_ref/libdumbref.so.
//
// Test infrastructure only: used by the parity tests (as the checker that pins the oracle) and by
// bench.py's reference arm (as the timed CPU baseline).  Nothing in the product links it.
//
// What it calls (reference file:line, relative to the DumbRay checkout):
//   Octree<Renderable<BakedTriFace>>::push/build   __source__/DataStructures/Objects/Scene/Raycasters/Octree/Octree.impl.cuh:97-129
//   Octree<...>::cast                              Octree.impl.cuh:174-212
//   DumbRenderer (CPU threads) via Renderer::iterate  __source__/DataStructures/Renderers/Renderer/Renderer.cu:143-156
//   DumbBasedShader / SimpleStochasticShader / FresnelShader / DefaultShader   __source__/DataStructures/Objects/Components/Shaders/*
//   SphericalLightEmitter / SimpleSoftDirectionalLight / SimpleDirectionalLight / Spotlight   __source__/DataStructures/Objects/Scene/Lights/*
//   DefaultPerspectiveLense / SimpleStochasticLense / Lenses::SphericalSegmentLense  __source__/DataStructures/Objects/Components/Lenses/*
#include "DataStructures/Renderers/DumbRenderer/DumbRenderer.cuh"
#include "ref_driver.h"
#include "DataStructures/Screen/FrameBuffer/BlockBasedFrameBuffer/BlockBasedFrameBuffer.cuh"
#include "DataStructures/Objects/Components/Shaders/DumbBasedShader/DumbBasedShader.cuh"
#include "DataStructures/Objects/Components/Shaders/SimpleStochasticShader/SimpleStochasticShader.cuh"
#include "DataStructures/Objects/Components/Lenses/DefaultPerspectiveLense/DefaultPerspectiveLense.cuh"
#include "DataStructures/Objects/Components/Lenses/SimpleStochasticLense/SimpleStochasticLense.cuh"
#include "DataStructures/Objects/Components/Lenses/SphericalSegmentLense/SphericalSegmentLense.cuh"
#include "DataStructures/Objects/Scene/Lights/SphericalLightEmitter/SphericalLightEmitter.cuh"
#include "DataStructures/Objects/Scene/Lights/SimpleSoftDirectionalLight/SimpleSoftDirectionalLight.cuh"
#include "DataStructures/Objects/Scene/Lights/SimpleDirectionalLight/SimpleDirectionalLight.cuh"
#include "DataStructures/Objects/Scene/Lights/Spotlight/Spotlight.cuh"
#include "DataStructures/Objects/Components/Shaders/FresnelShader/FresnelShader.cuh"
#include "DataStructures/Objects/Components/Shaders/DefaultShader/DefaultShader.cuh"
#include "Namespaces/Images/Images.cuh"
#include "Namespaces/Images/lodepng.h"
#include <cstring>
#include "Namespaces/MeshReader/MeshReader.h"
#include <thread>
#include <vector>
#include <chrono>

typedef Renderable<BakedTriFace> RefUnit;
typedef Octree<RefUnit> RefOctree;

static BakedTriFace make_face(const float *v, const float *n, const float *uv = NULL) {
	Triangle vert(Vector3(v[0], v[1], v[2]), Vector3(v[3], v[4], v[5]), Vector3(v[6], v[7], v[8]));
	Triangle norm;
	if (n != NULL) norm = Triangle(Vector3(n[0], n[1], n[2]), Vector3(n[3], n[4], n[5]), Vector3(n[6], n[7], n[8]));
	else {
		// Flat shading: the reference's outward normal is Triangle::normal() = (c-a)x(b-a).
		Vector3 fn = vert.normal().normalized();
		norm = Triangle(fn, fn, fn);
	}
	Triangle tex(Vector3(0, 0, 0), Vector3(1, 0, 0), Vector3(0, 1, 0));
	if (uv != NULL) tex = Triangle(Vector3(uv[0], uv[1], 0), Vector3(uv[2], uv[3], 0), Vector3(uv[4], uv[5], 0));
	return BakedTriFace(vert, norm, tex);
}

// Records of the reference objects the scene holds, built through their constructors.
//   material (48 floats): [0] 0 DumbBasedShader (fresnel [1..3], specular [4], diffuse [5..7],
//             metal [8]), 1 SimpleStochasticShader (colour [1..3], diffuse [4], smoothness [5],
//             shininess [6]), 2 Shaders::FresnelShader (colour [1..3]), 3 DefaultShader (as 1);
//             textures: [16..19] 1-based texture of the diffuse / fresnel / normal / alpha-cutout
//             ColoredTexture (0 = none; the Fresnel shader's colour is the first), [20..27] their
//             tilings, [28..35] offsets, [36..38] normal-map colour, [39] alpha-cutout threshold
//   light (16 floats):
//   light:    [0] 0 SphericalLightEmitter (colour [1..3], position [4..6], radius [7]),
//             1 SimpleSoftDirectionalLight (colour, direction [4..6], distance [7], softness [8]),
//             2 SimpleDirectionalLight (colour, direction, distance [7]),
//             3 Lights::Spotlight (colour, position [4..6], direction [7..9], luminosity [10], hotspot
//               [11] and falloff [12] angles, falloff power [13], emitter size [14], flags [15]:
//               1 emit from sphere, 2 cast shadows, samples << 2)
namespace {
// DumbBasedShader sets its alpha cutout only in fromDson; explicit instantiation (exempt from access
// checks) reaches the two members.
template <class Tag, typename Tag::type M>
struct RobRef {
	friend typename Tag::type get(Tag) { return M; }
};
struct RobCut { typedef ColoredTexture DumbBasedShader::*type; friend type get(RobCut); };
template struct RobRef<RobCut, &DumbBasedShader::alphaCutout>;
struct RobCutThr { typedef float DumbBasedShader::*type; friend type get(RobCutThr); };
template struct RobRef<RobCutThr, &DumbBasedShader::alphaCutoutThreshold>;

// Channel k of a material record as a ColoredTexture of colour c.
ColoredTexture channel(const float *m, int k, Color c) {
	const int t = (int)m[16 + k];
	if (t <= 0) return ColoredTexture(c);
	return ColoredTexture(c, t - 1, Vector2(m[20 + 2 * k], m[21 + 2 * k]), Vector2(m[28 + 2 * k], m[29 + 2 * k]));
}
}  // namespace

void ref_material(Material<BakedTriFace> &dst, const float *m) {
	const int type = (int)m[0];
	if (type == 0) {
		const Color white(1.0f, 1.0f, 1.0f, 1.0f);
		const ColoredTexture normal = channel(m, 2, Color(m[36], m[37], m[38], 1.0f));
		DumbBasedShader *d = dst.use<DumbBasedShader>(channel(m, 1, Color(m[1], m[2], m[3], 1.0f)), m[4],
			channel(m, 0, Color(m[5], m[6], m[7], 1.0f)), m[8], normal);
		if ((int)m[19] > 0) d->*get(RobCut()) = channel(m, 3, white);
		d->*get(RobCutThr()) = m[39];
	}
	else if (type == 1)
		dst.use<SimpleStochasticShader>(ColorRGB(m[1], m[2], m[3]), m[4], m[5], m[6]);
	else if (type == 2)
		dst.use<Shaders::FresnelShader>(channel(m, 0, Color(m[1], m[2], m[3], 1.0f)));
	else
		dst.use<DefaultShader>(ColorRGB(m[1], m[2], m[3]), m[4], m[5], m[6]);
}
void ref_light(Light &dst, const float *l) {
	const int type = (int)l[0];
	Color c(l[1], l[2], l[3], 1.0f);
	Vector3 v(l[4], l[5], l[6]);
	if (type == 0) dst.use<SphericalLightEmitter>(c, v, l[7]);
	else if (type == 1) dst.use<SimpleSoftDirectionalLight>(c, v, l[7], l[8]);
	else if (type == 2) dst.use<SimpleDirectionalLight>(c, v, l[7]);
	else {
		const int flags = (int)l[15];
		dst.use<Lights::Spotlight>(c, l[10], v, Vector3(l[7], l[8], l[9]), l[11], l[12], l[13], l[14],
			(flags & 1) != 0, (flags & 2) != 0, flags >> 2);
	}
}

extern "C" {

// Builds the reference octree over n triangles (xyz[9*n], optional per-vertex normals nrm[9*n],
// optional material ids).  Push order = triangle index, so hit index = hit.object - data.
void *dref_octree_create(const float *xyz, const float *nrm, const int *mat, int n) {
	RefOctree *tree = new RefOctree();
	for (int i = 0; i < n; i++)
		tree->push(RefUnit(make_face(xyz + 9 * i, (nrm != NULL) ? (nrm + 9 * i) : NULL), (mat != NULL) ? mat[i] : 0));
	tree->build();
	return (void *)tree;
}

int dref_octree_node_count(void *h) { return ((RefOctree *)h)->getNodeCount(); }

void dref_octree_destroy(void *h) { delete (RefOctree *)h; }

// Closest-hit casts of n rays (origins o[3n], directions d[3n]) with the reference's Octree::cast.
// idx = triangle index or -1, t = hitDistance (FLT_MAX on a miss).  Runs on `threads` host threads.
void dref_octree_cast(void *h, const float *o, const float *d, int n, int clip, int threads, int *idx, float *t) {
	const RefOctree *tree = (const RefOctree *)h;
	const RefUnit *base = (tree->getData() + 0);
	if (threads < 1) threads = 1;
	auto work = [&](int tid) {
		for (int i = tid; i < n; i += threads) {
			Ray r(Vector3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), Vector3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
			RaycastHit<RefUnit> hit;
			if (tree->cast(r, hit, clip != 0)) {
				idx[i] = (int)(hit.object - base);
				t[i] = hit.hitDistance;
			}
			else {
				idx[i] = -1;
				t[i] = FLT_MAX;
			}
		}
	};
	std::vector<std::thread> pool;
	for (int k = 1; k < threads; k++) pool.emplace_back(work, k);
	work(0);
	for (auto &th : pool) th.join();
}

// Material / light / lens records are flat float[16] arrays:
//   material: [0]=type (0 DumbBasedShader, 1 SimpleStochasticShader)
//     DumbBased: [1..3] fresnel rgb, [4] specular, [5..7] diffuse rgb, [8] metal
//     SimpleStochastic: [1..3] albedo rgb, [4] diffuse, [5] smoothness, [6] shininess
//   light: [0]=type (0 SphericalLightEmitter, 1 SimpleSoftDirectionalLight, 2 SimpleDirectionalLight)
//     Spherical: [1..3] color, [4..6] position, [7] radius
//     SoftDirectional: [1..3] color, [4..6] direction, [7] distance, [8] softness
//     Directional: [1..3] color, [4..6] direction, [7] distance
//   camera: [0]=lens (0 DefaultPerspectiveLense, 1 SimpleStochasticLense, 2 SphericalSegmentLense)
//     [1] angle (deg) / [1..2] alpha for spherical, [3] focal distance, [4] softness, [5..7] filter,
//     [8..10] position, [11..13] euler angles (deg)

// uv: per-corner texture coordinates float[n][3][2] or NULL (the fixed (0,0) (1,0) (0,1) corners).
void *dref_scene_create_uv(const float *xyz, const float *nrm, const float *uv, const int *mat, int n,
                           const float *mats, int n_mats, const float *lights, int n_lights, const float *cam) {
	RefScene *s = new RefScene();
	s->scene.materials.cpuHandle()->flush(n_mats);
	for (int i = 0; i < n_mats; i++) {
		const float *m = mats + 48 * i;
		Material<BakedTriFace> &dst = s->scene.materials.cpuHandle()->operator[](i);
		ref_material(dst, m);
	}
	s->scene.lights.cpuHandle()->flush(n_lights);
	for (int i = 0; i < n_lights; i++) {
		const float *l = lights + 16 * i;
		ref_light(s->scene.lights.cpuHandle()->operator[](i), l);
	}
	int lens = (int)cam[0];
	if (lens == 0) s->camera.cpuHandle()->lense.use<DefaultPerspectiveLense>(cam[1]);
	else if (lens == 1) s->camera.cpuHandle()->lense.use<SimpleStochasticLense>(cam[1]);
	else s->camera.cpuHandle()->lense.use<Lenses::SphericalSegmentLense>(Vector2(cam[1], cam[2]), cam[3], cam[4], Color(cam[5], cam[6], cam[7], 1.0f));
	s->camera.cpuHandle()->transform = Transform(Vector3(cam[8], cam[9], cam[10]), Vector3(cam[11], cam[12], cam[13]), Vector3(1.0f, 1.0f, 1.0f));
	RefOctree *tree = s->scene.geometry.cpuHandle();
	for (int i = 0; i < n; i++)
		tree->push(RefUnit(make_face(xyz + 9 * i, (nrm != NULL) ? (nrm + 9 * i) : NULL, (uv != NULL) ? (uv + 6 * i) : NULL),
			(mat != NULL) ? mat[i] : 0));
	tree->build();
	return (void *)s;
}

void *dref_scene_create(const float *xyz, const float *nrm, const int *mat, int n,
                        const float *mats, int n_mats, const float *lights, int n_lights, const float *cam) {
	return dref_scene_create_uv(xyz, nrm, NULL, mat, n, mats, n_mats, lights, n_lights, cam);
}

// The scene's textures: texture t is width whf[3t] x height whf[3t+1] with Texture::Filtering
// whf[3t+2], texels rgba[t] (float[h][w][4], row 0 first).
void dref_scene_set_textures(void *h, int n, const int *whf, const float *const *rgba) {
	RefScene *s = (RefScene *)h;
	Stacktor<Texture> *tex = s->scene.textures.cpuHandle();
	tex->clear();
	tex->flush(n);
	for (int t = 0; t < n; t++) {
		Texture &x = (*tex)[t];
		const int w = whf[3 * t], hh = whf[3 * t + 1];
		x.setReolution((uint32_t)w, (uint32_t)hh);
		x.setFiltering((Texture::Filtering)whf[3 * t + 2]);
		for (int y = 0; y < hh; y++)
			for (int xx = 0; xx < w; xx++) {
				const float *p = rgba[t] + 4 * ((size_t)y * w + xx);
				x((uint32_t)xx, (uint32_t)y) = Color(p[0], p[1], p[2], p[3]);
			}
	}
}

void dref_scene_destroy(void *h) { delete (RefScene *)h; }

// Renders `iterations` progressive iterations with the reference DumbRenderer on `threads` CPU
// threads (BlockBuffer = 8x16 blocks) and writes the blended float4 image row-major to rgba[4*W*H].
// Returns the wall time of the iterations in seconds (scene build excluded), or -1 on failure.
double dref_render(void *h, int width, int height, int fsaa_x, int fsaa_y, int max_bounces,
                   int cull_backfaces, int iterations, int threads, float *rgba) {
	RefScene *s = (RefScene *)h;
	FrameBufferManager fb;
	fb.cpuHandle()->use<BlockBuffer>();
	if (!fb.cpuHandle()->setResolution(width, height)) return -1.0;
	DumbRenderer renderer(Renderer::ThreadConfiguration::cpuOnly(threads), BlockRenderer::BlockConfiguration(),
		&fb, &s->scene, &s->camera, DumbRenderer::BOXING_MODE_HEIGHT_BASED, max_bounces, fsaa_x, fsaa_y, 1, cull_backfaces != 0);
	auto t0 = std::chrono::steady_clock::now();
	for (int i = 0; i < iterations; i++)
		if (!renderer.iterate()) return -1.0;
	auto t1 = std::chrono::steady_clock::now();
	if (rgba != NULL) {
		for (int y = 0; y < height; y++)
			for (int x = 0; x < width; x++) {
				Color c = fb.cpuHandle()->getColor(x, y);
				float *p = rgba + 4 * (y * width + x);
				p[0] = c.r; p[1] = c.g; p[2] = c.b; p[3] = c.a;
			}
	}
	return std::chrono::duration<double>(t1 - t0).count();
}

// OBJ files through the reference's MeshReader::readObj + PolyMesh::bake: a handle holding the
// meshes and names, then per mesh the baked triangles (vert / norm / tex corners, 9 floats each).
struct RefObj {
	Stacktor<PolyMesh> meshes;
	Stacktor<String> names;
};
void *dref_obj_read(const char *path) {
	RefObj *o = new RefObj();
	if (!MeshReader::readObj(o->meshes, o->names, path)) { delete o; return NULL; }
	return o;
}
int dref_obj_meshes(void *h) { return ((RefObj *)h)->meshes.size(); }
int dref_obj_names(void *h) { return ((RefObj *)h)->names.size(); }
const char *dref_obj_name(void *h, int i) { return ((RefObj *)h)->names[i] + 0; }
int dref_obj_triangles(void *h, int i, float *xyz, float *nrm, float *uv) {
	const BakedTriMesh m = ((RefObj *)h)->meshes[i].bake();
	for (int k = 0; k < m.size(); k++) {
		const Triangle *t[3] = {&m[k].vert, &m[k].norm, &m[k].tex};
		float *dst[3] = {xyz, nrm, uv};
		for (int q = 0; q < 3; q++) {
			if (dst[q] == NULL) continue;
			const Vertex *c[3] = {&t[q]->a, &t[q]->b, &t[q]->c};
			for (int v = 0; v < 3; v++) {
				dst[q][9 * k + 3 * v] = c[v]->x; dst[q][9 * k + 3 * v + 1] = c[v]->y; dst[q][9 * k + 3 * v + 2] = c[v]->z;
			}
		}
	}
	return m.size();
}
void dref_obj_free(void *h) { delete (RefObj *)h; }

// Writes a row-major float4 image through the reference's own Images::saveBufferPNG (lodepng), via
// a host BlockBuffer filled with FrameBuffer::setColor.  Returns the Images::Error code (0 = ok).
// lodepng::decode to 8-bit RGBA (what Images::getTexturePNG decodes textures with): returns the
// lodepng error code (0 = success), writes width / height and, when rgba8 is not NULL, the pixels.
int dref_png_decode(const char *path, int *width, int *height, unsigned char *rgba8) {
	std::vector<unsigned char> px;
	unsigned int w = 0, h = 0;
	unsigned int err = lodepng::decode(px, w, h, std::string(path));
	*width = (int)w;
	*height = (int)h;
	if (!err && rgba8 != NULL) std::memcpy(rgba8, px.data(), px.size());
	return (int)err;
}

int dref_save_png(const float *rgba, int width, int height, const char *path) {
	FrameBufferManager fb;
	fb.cpuHandle()->use<BlockBuffer>();
	if (!fb.cpuHandle()->setResolution(width, height)) return -1;
	for (int y = 0; y < height; y++)
		for (int x = 0; x < width; x++) {
			const float *p = rgba + 4 * (y * width + x);
			fb.cpuHandle()->setColor(x, y, Color(p[0], p[1], p[2], p[3]));
		}
	return (int)Images::saveBufferPNG(*fb.cpuHandle(), path);
}

}  // extern "C"
