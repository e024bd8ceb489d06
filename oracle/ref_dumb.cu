// The reference's own scene-file loader (DumbRenderContext::fromFile and everything it calls),
// wrapped in a C ABI that reports what it built: the pushed triangles, material / light / lens
// parameters, the camera transform and the renderer settings.  Test infrastructure only (the
// checker for the product's .dumb loader); nothing in the product links it.
//
// DumbRenderContext.cu keeps its parsed state in a struct inside an unnamed namespace and a private
// `void *data` member, and the shaders and lenses keep their parameters private.  So this file
// includes that translation unit textually (its unnamed-namespace types become visible here; the
// build compiles it through this file only) and reads the private members through explicit
// template instantiation, which the language exempts from access checking.  The reference sources
// are not modified.
//
// What it calls (reference file:line, relative to the DumbRay checkout):
//   DumbRenderContext::fromFile / fromDson          __source__/DataStructures/DumbRenderContext/DumbRenderContext.cu:300-372
//   parseMaterial / parseLight / parseCamera / parseRenderer / parseObject
//                                                   DumbRenderContext.cu:488-727, 754-820
//   Transform::fromDson / rebake                    __source__/DataStructures/Objects/Components/Transform/Transform.impl.h:209-281
//   DumbBasedShader / SimpleStochasticShader ::fromDson, lights and lenses ::fromDson
#include <string>
#include <sstream>
#include <fstream>
#include <iomanip>
#include <vector>
#include <mutex>
#include <set>
#include <map>
#include <unordered_map>
#include <thread>
#include <chrono>
#include <cstring>

#include "DataStructures/DumbRenderContext/DumbRenderContext.cu"
#include "DataStructures/Objects/Components/Shaders/DumbBasedShader/DumbBasedShader.cuh"
#include "DataStructures/Objects/Components/Shaders/SimpleStochasticShader/SimpleStochasticShader.cuh"
#include "DataStructures/Objects/Components/Lenses/SimpleStochasticLense/SimpleStochasticLense.cuh"
#include "DataStructures/Objects/Components/Lenses/SphericalSegmentLense/SphericalSegmentLense.cuh"
#include "DataStructures/Objects/Scene/Lights/SphericalLightEmitter/SphericalLightEmitter.cuh"
#include "DataStructures/Objects/Scene/Lights/SimpleSoftDirectionalLight/SimpleSoftDirectionalLight.cuh"
#include "DataStructures/Objects/Components/Lenses/DefaultPerspectiveLense/DefaultPerspectiveLense.cuh"
#include "DataStructures/Objects/Components/Shaders/FresnelShader/FresnelShader.cuh"
#include "DataStructures/Objects/Components/Shaders/DefaultShader/DefaultShader.cuh"
#include "DataStructures/Objects/Scene/Lights/Spotlight/Spotlight.cuh"
#include "DataStructures/Objects/Scene/Lights/SimpleDirectionalLight/SimpleDirectionalLight.cuh"
#include "DataStructures/Screen/FrameBuffer/BlockBasedFrameBuffer/BlockBasedFrameBuffer.cuh"

// Reference objects from records (oracle/ref_driver.cu).
void ref_material(Material<BakedTriFace> &dst, const float *m);
void ref_light(Light &dst, const float *l);

namespace {

// Private member access by explicit instantiation.
template <class Tag, typename Tag::type M>
struct Rob {
	friend typename Tag::type get(Tag) { return M; }
};
#define DREF_ROB(NAME, CLASS, TYPE, MEMBER) \
	struct NAME { typedef TYPE CLASS::*type; friend type get(NAME); }; \
	template struct Rob<NAME, &CLASS::MEMBER>;

DREF_ROB(RobData, DumbRenderContext, void *, data)
DREF_ROB(RobFresnel, DumbBasedShader, ColoredTexture, fresnelColor)
DREF_ROB(RobDiffuse, DumbBasedShader, ColoredTexture, diffuseColor)
DREF_ROB(RobNormal, DumbBasedShader, ColoredTexture, normalColor)
DREF_ROB(RobAlpha, DumbBasedShader, ColoredTexture, alphaCutout)
DREF_ROB(RobAlphaThr, DumbBasedShader, float, alphaCutoutThreshold)
DREF_ROB(RobSpec, DumbBasedShader, float, spec)
DREF_ROB(RobSpecMass, DumbBasedShader, float, specMass)
DREF_ROB(RobAlbedo, SimpleStochasticShader, ColorRGB, albedo)
DREF_ROB(RobDiff, SimpleStochasticShader, float, diff)
DREF_ROB(RobGloss, SimpleStochasticShader, float, gloss)
DREF_ROB(RobShine, SimpleStochasticShader, float, shine)
DREF_ROB(RobStochX, SimpleStochasticLense, float, x)
DREF_ROB(RobPerspX, DefaultPerspectiveLense, float, x)
DREF_ROB(RobSegAlpha, Lenses::SphericalSegmentLense, Vector2, alpha)
DREF_ROB(RobSegDist, Lenses::SphericalSegmentLense, float, dist)
DREF_ROB(RobSegSoft, Lenses::SphericalSegmentLense, float, soft)
DREF_ROB(RobSegFilter, Lenses::SphericalSegmentLense, Color, filter)
DREF_ROB(RobFresnelColor, Shaders::FresnelShader, ColoredTexture, color)
DREF_ROB(RobDefAlbedo, DefaultShader, ColorRGB, albedo)
DREF_ROB(RobDefDiff, DefaultShader, float, diff)
DREF_ROB(RobDefGloss, DefaultShader, float, gloss)
DREF_ROB(RobDefShine, DefaultShader, float, shininess)
DREF_ROB(RobSpotColor, Lights::Spotlight, Color, color)
DREF_ROB(RobSpotPos, Lights::Spotlight, Vector3, position)
DREF_ROB(RobSpotDir, Lights::Spotlight, Vector3, direction)
DREF_ROB(RobSpotEmit, Lights::Spotlight, float, emitterSize)
DREF_ROB(RobSpotInner, Lights::Spotlight, float, innerCosine)
DREF_ROB(RobSpotOuter, Lights::Spotlight, float, outerCosine)
DREF_ROB(RobSpotFalloff, Lights::Spotlight, float, outerFalloff)
DREF_ROB(RobSpotFlags, Lights::Spotlight, uint8_t, flags)

DumbRenderContextData *ctx_data(DumbRenderContext *c) { return (DumbRenderContextData *)(c->*get(RobData())); }

// Type of a function-pack object: compare its function pointers with a probe's.
template <class Pack, class Generic_, class Type>
bool is_type(const Generic_ &g) {
	Generic_ probe;
	probe.template use<Type>();
	return std::memcmp(&g.functions(), &probe.functions(), sizeof(Pack)) == 0;
}

// Canonical dumps; the same layout for both sides of the comparison.
//   material (float[48]): [0]=type (0 DumbBasedShader, 1 SimpleStochasticShader, -1 other)
//     DumbBased: [1..3] fresnelColor, [4..6] diffuseColor (constructor-scaled), [7] spec,
//       [8] specMass, [9] alphaCutoutThreshold, [10..13] texture ids fresnel/diffuse/normal/alpha,
//       [16..35] those four channels' (id, tiling, offset), [36..38] normal colour, [39..42] cutout colour
//     SimpleStochastic: [1..3] albedo, [4] diff, [5] gloss, [6] shine
//     (2) FresnelShader: [1..3] colour, [4] texture id, [16..20] (id, tiling, offset);  (3) DefaultShader: [1..3] albedo, [4] diff,
//       [5] gloss, [6] shininess
// Texture channel c of a ColoredTexture into o: [0] texture id, [1..2] tiling, [3..4] offset.
void dump_channel(const ColoredTexture &c, float *o) {
	o[0] = (float)c.textureId;
	o[1] = c.tiling.x; o[2] = c.tiling.y; o[3] = c.offset.x; o[4] = c.offset.y;
}
void dump_material(const Material<BakedTriFace> &m, float *o) {
	std::memset(o, 0, 48 * sizeof(float));
	typedef Shader<BakedTriFace> Pack;
	if (is_type<Pack, Material<BakedTriFace>, DumbBasedShader>(m)) {
		const DumbBasedShader *s = m.getObject<DumbBasedShader>();
		const ColoredTexture &f = s->*get(RobFresnel()), &d = s->*get(RobDiffuse());
		o[0] = 0;
		o[1] = f.color.r; o[2] = f.color.g; o[3] = f.color.b;
		o[4] = d.color.r; o[5] = d.color.g; o[6] = d.color.b;
		o[7] = s->*get(RobSpec()); o[8] = s->*get(RobSpecMass()); o[9] = s->*get(RobAlphaThr());
		o[10] = (float)f.textureId; o[11] = (float)d.textureId;
		o[12] = (float)(s->*get(RobNormal())).textureId; o[13] = (float)(s->*get(RobAlpha())).textureId;
		const ColoredTexture &nc = s->*get(RobNormal()), &ac = s->*get(RobAlpha());
		dump_channel(f, o + 16); dump_channel(d, o + 21); dump_channel(nc, o + 26); dump_channel(ac, o + 31);
		o[36] = nc.color.r; o[37] = nc.color.g; o[38] = nc.color.b;
		o[39] = ac.color.r; o[40] = ac.color.g; o[41] = ac.color.b; o[42] = ac.color.a;
	} else if (is_type<Pack, Material<BakedTriFace>, SimpleStochasticShader>(m)) {
		const SimpleStochasticShader *s = m.getObject<SimpleStochasticShader>();
		const ColorRGB &a = s->*get(RobAlbedo());
		o[0] = 1;
		o[1] = a.r; o[2] = a.g; o[3] = a.b;
		o[4] = s->*get(RobDiff()); o[5] = s->*get(RobGloss()); o[6] = s->*get(RobShine());
	} else if (is_type<Pack, Material<BakedTriFace>, Shaders::FresnelShader>(m)) {
		const ColoredTexture &c = m.getObject<Shaders::FresnelShader>()->*get(RobFresnelColor());
		o[0] = 2;
		o[1] = c.color.r; o[2] = c.color.g; o[3] = c.color.b; o[4] = (float)c.textureId;
		dump_channel(c, o + 16);
	} else if (is_type<Pack, Material<BakedTriFace>, DefaultShader>(m)) {
		const DefaultShader *s = m.getObject<DefaultShader>();
		const ColorRGB &a = s->*get(RobDefAlbedo());
		o[0] = 3;
		o[1] = a.r; o[2] = a.g; o[3] = a.b;
		o[4] = s->*get(RobDefDiff()); o[5] = s->*get(RobDefGloss()); o[6] = s->*get(RobDefShine());
	} else o[0] = -1;
}
//   light: [0]=type (0 SphericalLightEmitter, 1 SimpleSoftDirectionalLight, 3 Lights::Spotlight, -1 other)
//     spherical: [1..3] col, [4..6] pos, [7] rad;  soft directional: [1..3] color, [4..6] dir, [7] dist, [8] soft
//     spotlight: [1..3] color (x luminosity), [4..6] position, [7..9] direction, [10] emitterSize,
//       [11] innerCosine, [12] outerCosine, [13] outerFalloff, [14] flags
void dump_light(const Light &l, float *o) {
	std::memset(o, 0, 16 * sizeof(float));
	if (is_type<LightInterface, Light, SphericalLightEmitter>(l)) {
		const SphericalLightEmitter *s = l.getObject<SphericalLightEmitter>();
		o[0] = 0;
		o[1] = s->col.r; o[2] = s->col.g; o[3] = s->col.b;
		o[4] = s->pos.x; o[5] = s->pos.y; o[6] = s->pos.z; o[7] = s->rad;
	} else if (is_type<LightInterface, Light, SimpleSoftDirectionalLight>(l)) {
		const SimpleSoftDirectionalLight *s = l.getObject<SimpleSoftDirectionalLight>();
		o[0] = 1;
		o[1] = s->color.r; o[2] = s->color.g; o[3] = s->color.b;
		o[4] = s->dir.x; o[5] = s->dir.y; o[6] = s->dir.z; o[7] = s->dist; o[8] = s->soft;
	} else if (is_type<LightInterface, Light, Lights::Spotlight>(l)) {
		const Lights::Spotlight *s = l.getObject<Lights::Spotlight>();
		const Color &c = s->*get(RobSpotColor());
		const Vector3 &p = s->*get(RobSpotPos()), &d = s->*get(RobSpotDir());
		o[0] = 3;
		o[1] = c.r; o[2] = c.g; o[3] = c.b;
		o[4] = p.x; o[5] = p.y; o[6] = p.z; o[7] = d.x; o[8] = d.y; o[9] = d.z;
		o[10] = s->*get(RobSpotEmit()); o[11] = s->*get(RobSpotInner()); o[12] = s->*get(RobSpotOuter());
		o[13] = s->*get(RobSpotFalloff()); o[14] = (float)(s->*get(RobSpotFlags()));
	} else o[0] = -1;
}
//   lens: [0]=type (0 DefaultPerspectiveLense, 1 SimpleStochasticLense, 2 SphericalSegmentLense, -1 other/none)
//     perspective / stochastic: [1] x;  spherical segment: [1..2] alpha, [3] dist, [4] soft, [5..7] filter
void dump_lens(const Lense &l, float *o) {
	std::memset(o, 0, 8 * sizeof(float));
	if (l.object() == NULL) { o[0] = -1; return; }
	if (is_type<LenseFunctionPack, Lense, DefaultPerspectiveLense>(l)) {
		o[0] = 0; o[1] = l.getObject<DefaultPerspectiveLense>()->*get(RobPerspX());
	} else if (is_type<LenseFunctionPack, Lense, SimpleStochasticLense>(l)) {
		o[0] = 1; o[1] = l.getObject<SimpleStochasticLense>()->*get(RobStochX());
	} else if (is_type<LenseFunctionPack, Lense, Lenses::SphericalSegmentLense>(l)) {
		const Lenses::SphericalSegmentLense *s = l.getObject<Lenses::SphericalSegmentLense>();
		const Vector2 &a = s->*get(RobSegAlpha());
		const Color &f = s->*get(RobSegFilter());
		o[0] = 2; o[1] = a.x; o[2] = a.y; o[3] = s->*get(RobSegDist()); o[4] = s->*get(RobSegSoft());
		o[5] = f.r; o[6] = f.g; o[7] = f.b;
	} else o[0] = -1;
}
//   transform (float[15]): [0..2] right(), [3..5] up(), [6..8] front() (Transform::direction basis),
//     [9..17] rows of the point transform (v >> t = (v.row_x, v.row_y, v.row_z) + position),
//     [18..20] position
void dump_transform(const Transform &t, float *o) {
	Vector3 r = t.right(), u = t.up(), f = t.front();
	o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = u.x; o[4] = u.y; o[5] = u.z; o[6] = f.x; o[7] = f.y; o[8] = f.z;
	Transform z = t;
	z.setPosition(Vector3(0.0f, 0.0f, 0.0f));
	Vector3 cx = Vector3(1.0f, 0.0f, 0.0f) >> z, cy = Vector3(0.0f, 1.0f, 0.0f) >> z, cz = Vector3(0.0f, 0.0f, 1.0f) >> z;
	// cx = (row_x.x, row_y.x, row_z.x) etc.
	o[9] = cx.x; o[10] = cy.x; o[11] = cz.x;
	o[12] = cx.y; o[13] = cy.y; o[14] = cz.y;
	o[15] = cx.z; o[16] = cy.z; o[17] = cz.z;
	const Vector3 &p = t.getPosition();
	o[18] = p.x; o[19] = p.y; o[20] = p.z;
}

struct RefDumb {
	DumbRenderContext ctx;
	std::string error;
};

}  // namespace

extern "C" {

// Loads a scene file with the reference's loader.  Returns NULL on failure and copies the loader's
// error text into err (err_len bytes, NUL-terminated).
void *dref_dumb_load(const char *path, char *err, int err_len) {
	RefDumb *h = new RefDumb();
	std::stringstream es;
	bool ok = h->ctx.fromFile(path, &es);
	if (err != NULL && err_len > 0) {
		std::string e = es.str();
		std::strncpy(err, e.c_str(), (size_t)err_len - 1);
		err[err_len - 1] = 0;
	}
	if (!ok) { delete h; return NULL; }
	return h;
}
void dref_dumb_free(void *h) { delete (RefDumb *)h; }

// counts: [0] triangles, [1] materials, [2] lights
void dref_dumb_counts(void *h, int *counts) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	counts[0] = d->scene.geometry.cpuHandle()->getData().size();
	counts[1] = d->scene.materials.cpuHandle()->size();
	counts[2] = d->scene.lights.cpuHandle()->size();
}

// Pushed triangles in push order: vertices, normals (9 floats each) and material ids.
void dref_dumb_geometry(void *h, float *xyz, float *nrm, int *mat) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	const Stacktor<Renderable<BakedTriFace> > &units = d->scene.geometry.cpuHandle()->getData();
	for (int i = 0; i < units.size(); i++) {
		const BakedTriFace &f = units[i].object;
		const Vector3 *v[3] = { &f.vert.a, &f.vert.b, &f.vert.c };
		const Vector3 *n[3] = { &f.norm.a, &f.norm.b, &f.norm.c };
		for (int k = 0; k < 3; k++) {
			xyz[9 * i + 3 * k] = v[k]->x; xyz[9 * i + 3 * k + 1] = v[k]->y; xyz[9 * i + 3 * k + 2] = v[k]->z;
			nrm[9 * i + 3 * k] = n[k]->x; nrm[9 * i + 3 * k + 1] = n[k]->y; nrm[9 * i + 3 * k + 2] = n[k]->z;
		}
		mat[i] = units[i].materialId;
	}
}

// Texture coordinates of the pushed triangles (tex corners x, y): uv[n][3][2].
void dref_dumb_texcoords(void *h, float *uv) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	const Stacktor<Renderable<BakedTriFace> > &units = d->scene.geometry.cpuHandle()->getData();
	for (int i = 0; i < units.size(); i++) {
		const Triangle &t = units[i].object.tex;
		const Vector3 *c[3] = { &t.a, &t.b, &t.c };
		for (int k = 0; k < 3; k++) { uv[6 * i + 2 * k] = c[k]->x; uv[6 * i + 2 * k + 1] = c[k]->y; }
	}
}
// Texture count, then texture i's size, filtering and texels (float[h][w][4]) when rgba is not NULL.
int dref_dumb_texture_count(void *h) { return ctx_data(&((RefDumb *)h)->ctx)->scene.textures.cpuHandle()->size(); }
void dref_dumb_texture(void *h, int i, int *whf, float *rgba) {
	const Texture &t = (*ctx_data(&((RefDumb *)h)->ctx)->scene.textures.cpuHandle())[i];
	whf[0] = (int)t.width(); whf[1] = (int)t.height(); whf[2] = (int)t.filtering();
	if (rgba == NULL) return;
	for (uint32_t y = 0; y < t.height(); y++)
		for (uint32_t x = 0; x < t.width(); x++) {
			const Color &c = t(x, y);
			float *p = rgba + 4 * ((size_t)y * t.width() + x);
			p[0] = c.r; p[1] = c.g; p[2] = c.b; p[3] = c.a;
		}
}

void dref_dumb_material(void *h, int i, float *out) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	dump_material((*d->scene.materials.cpuHandle())[i], out);  // float[48]
}
void dref_dumb_light(void *h, int i, float *out) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	dump_light((*d->scene.lights.cpuHandle())[i], out);
}
// camera: [0..7] lens dump, [8..28] transform dump
void dref_dumb_camera(void *h, float *out) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	const Camera *c = d->camera.cpuHandle();
	dump_lens(c->lense, out);
	dump_transform(c->transform, out + 8);
}
// settings: [0] boxing mode, [1] max bounces, [2..3] samples per pixel x/y, [4] pixels per GPU
// thread, [5] ignore backfaces
void dref_dumb_settings(void *h, int *out) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	out[0] = (int)d->rendererSettings.boxingMode;
	out[1] = d->rendererSettings.maxBounces;
	out[2] = d->rendererSettings.samplesPerPixelX;
	out[3] = d->rendererSettings.samplesPerPixelY;
	out[4] = d->rendererSettings.pixelsPerGPUThread;
	out[5] = d->rendererSettings.ignoreBackfaces ? 1 : 0;
}

// The same dumps for objects built from constructor arguments (the records dref_scene_create takes),
// so a loader's output can be compared with the reference's field by field.
void dref_record_material(const float *m, float *out) {
	Material<BakedTriFace> mat;
	ref_material(mat, m);
	dump_material(mat, out);
}
void dref_record_light(const float *l, float *out) {
	Light light;
	ref_light(light, l);
	dump_light(light, out);
}
void dref_record_lens(const float *cam, float *out) {
	Lense lense;
	int lens = (int)cam[0];
	if (lens == 0) lense.use<DefaultPerspectiveLense>(cam[1]);
	else if (lens == 1) lense.use<SimpleStochasticLense>(cam[1]);
	else lense.use<Lenses::SphericalSegmentLense>(Vector2(cam[1], cam[2]), cam[3], cam[4], Color(cam[5], cam[6], cam[7], 1.0f));
	dump_lens(lense, out);
}

// Renders the loaded scene with the reference DumbRenderer on `threads` CPU threads using the
// file's camera and renderer settings (builds the octree on first use); rgba[4*W*H] row-major.
// Returns the wall time of the iterations in seconds, or -1 on failure.
double dref_dumb_render(void *h, int width, int height, int iterations, int threads, float *rgba) {
	DumbRenderContextData *d = ctx_data(&((RefDumb *)h)->ctx);
	if (d->scene.geometry.cpuHandle()->getNodeCount() <= 0) d->scene.geometry.cpuHandle()->build();
	FrameBufferManager fb;
	fb.cpuHandle()->use<BlockBuffer>();
	if (!fb.cpuHandle()->setResolution(width, height)) return -1.0;
	DumbRenderContextData::RendererSettings &s = d->rendererSettings;
	DumbRenderer renderer(Renderer::ThreadConfiguration::cpuOnly(threads), BlockRenderer::BlockConfiguration(),
		&fb, &d->scene, &d->camera, s.boxingMode, s.maxBounces, s.samplesPerPixelX, s.samplesPerPixelY,
		1, s.ignoreBackfaces);
	auto t0 = std::chrono::steady_clock::now();
	for (int i = 0; i < iterations; i++)
		if (!renderer.iterate()) return -1.0;
	auto t1 = std::chrono::steady_clock::now();
	for (int y = 0; y < height; y++)
		for (int x = 0; x < width; x++) {
			Color c = fb.cpuHandle()->getColor(x, y);
			float *p = rgba + 4 * (y * width + x);
			p[0] = c.r; p[1] = c.g; p[2] = c.b; p[3] = c.a;
		}
	return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
