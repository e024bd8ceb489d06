// GB300Renderer.cu - see GB300Renderer.cuh.
//
// Reading the reference objects: the shaders, lenses and the Spotlight keep their constructor
// state in private members, and a device frame buffer's pixel pointer sits in BlockBufferData's
// private registry of device mirrors.  A maintainer adding this file to the DumbRay tree would give
// those classes public getters; compiled from outside the tree, it reads them through pointers to
// members named in explicit template instantiations (which the language exempts from access checks),
// so the reference sources stay unmodified.
#include "GB300Renderer.cuh"

#include <cmath>
#include <cstring>
#include <unordered_map>

#include "DataStructures/Objects/Components/Shaders/DumbBasedShader/DumbBasedShader.cuh"
#include "DataStructures/Objects/Components/Shaders/SimpleStochasticShader/SimpleStochasticShader.cuh"
#include "DataStructures/Objects/Components/Shaders/FresnelShader/FresnelShader.cuh"
#include "DataStructures/Objects/Components/Shaders/DefaultShader/DefaultShader.cuh"
#include "DataStructures/Objects/Components/Lenses/DefaultPerspectiveLense/DefaultPerspectiveLense.cuh"
#include "DataStructures/Objects/Components/Lenses/SimpleStochasticLense/SimpleStochasticLense.cuh"
#include "DataStructures/Objects/Components/Lenses/SphericalSegmentLense/SphericalSegmentLense.cuh"
#include "DataStructures/Objects/Scene/Lights/SphericalLightEmitter/SphericalLightEmitter.cuh"
#include "DataStructures/Objects/Scene/Lights/SimpleSoftDirectionalLight/SimpleSoftDirectionalLight.cuh"
#include "DataStructures/Objects/Scene/Lights/SimpleDirectionalLight/SimpleDirectionalLight.cuh"
#include "DataStructures/Objects/Scene/Lights/Spotlight/Spotlight.cuh"
#include "DataStructures/Screen/FrameBuffer/BlockBasedFrameBuffer/BlockBasedFrameBuffer.cuh"

namespace {

// ---- private-member access ---------------------------------------------------------------------
// Member<Key>::ptr is set by the explicit instantiation Bind<Key, &Class::member>.
template <class Key>
struct Member {
	static typename Key::type ptr;
};
template <class Key>
typename Key::type Member<Key>::ptr;
template <class Key, typename Key::type P>
struct Bind {
	struct Setter {
		Setter() { Member<Key>::ptr = P; }
	};
	static Setter setter;
};
template <class Key, typename Key::type P>
typename Bind<Key, P>::Setter Bind<Key, P>::setter;

#define GB300_MEMBER(KEY, CLASS, TYPE, NAME)            \
	struct KEY {                                        \
		typedef TYPE CLASS::*type;                      \
	};                                                  \
	template struct Bind<KEY, &CLASS::NAME>;
#define GB300_STATIC(KEY, CLASS, TYPE, NAME)            \
	struct KEY {                                        \
		typedef TYPE *type;                             \
	};                                                  \
	template struct Bind<KEY, &CLASS::NAME>;

GB300_MEMBER(DbFresnel, DumbBasedShader, ColoredTexture, fresnelColor)
GB300_MEMBER(DbDiffuse, DumbBasedShader, ColoredTexture, diffuseColor)
GB300_MEMBER(DbNormal, DumbBasedShader, ColoredTexture, normalColor)
GB300_MEMBER(DbAlpha, DumbBasedShader, ColoredTexture, alphaCutout)
GB300_MEMBER(DbAlphaThreshold, DumbBasedShader, float, alphaCutoutThreshold)
GB300_MEMBER(DbSpec, DumbBasedShader, float, spec)
GB300_MEMBER(DbMetal, DumbBasedShader, float, specMass)
GB300_MEMBER(SsAlbedo, SimpleStochasticShader, ColorRGB, albedo)
GB300_MEMBER(SsDiffuse, SimpleStochasticShader, float, diff)
GB300_MEMBER(SsGloss, SimpleStochasticShader, float, gloss)
GB300_MEMBER(SsShine, SimpleStochasticShader, float, shine)
GB300_MEMBER(FrColor, Shaders::FresnelShader, ColoredTexture, color)
GB300_MEMBER(DfAlbedo, DefaultShader, ColorRGB, albedo)
GB300_MEMBER(DfDiffuse, DefaultShader, float, diff)
GB300_MEMBER(DfGloss, DefaultShader, float, gloss)
GB300_MEMBER(DfShine, DefaultShader, float, shininess)
GB300_MEMBER(SpColor, Lights::Spotlight, Color, color)
GB300_MEMBER(SpPosition, Lights::Spotlight, Vertex, position)
GB300_MEMBER(SpDirection, Lights::Spotlight, Vector3, direction)
GB300_MEMBER(SpEmitter, Lights::Spotlight, float, emitterSize)
GB300_MEMBER(SpInner, Lights::Spotlight, float, innerCosine)
GB300_MEMBER(SpOuter, Lights::Spotlight, float, outerCosine)
GB300_MEMBER(SpFalloff, Lights::Spotlight, float, outerFalloff)
GB300_MEMBER(SpFlags, Lights::Spotlight, uint8_t, flags)
GB300_MEMBER(PerspX, DefaultPerspectiveLense, float, x)
GB300_MEMBER(StochX, SimpleStochasticLense, float, x)
GB300_MEMBER(SegAlpha, Lenses::SphericalSegmentLense, Vector2, alpha)
GB300_MEMBER(SegDist, Lenses::SphericalSegmentLense, float, dist)
GB300_MEMBER(SegSoft, Lenses::SphericalSegmentLense, float, soft)
GB300_MEMBER(SegFilter, Lenses::SphericalSegmentLense, Color, filter)
GB300_MEMBER(BbData, BlockBufferData, Color *, data)
typedef std::unordered_map<const void *, BlockBufferData> MirrorMap;
GB300_STATIC(BbMirrors, BlockBufferData, MirrorMap, deviceReferenceMirrors)
GB300_STATIC(BbLock, BlockBufferData, std::mutex, deviceReferenceLock)

template <class Key, class Object>
auto &field(Object &o) { return o.*Member<Key>::ptr; }

// Which shader / lens / light a function-pack object holds: its function pointers equal those of
// a probe object of that type (constructed from `args`).
template <class Type, class Holder, class... Args>
bool holds(const Holder &h, const Args &...args) {
	Holder probe;
	probe.template use<Type>(args...);
	return std::memcmp(&h.functions(), &probe.functions(), sizeof(h.functions())) == 0;
}

const float kRadian = 57.29577951308233f;   // RADIAN, Vector3.h

void set3(float *d, float x, float y, float z) { d[0] = x; d[1] = y; d[2] = z; }

// ColoredTexture channel k of a material: colour into rgb (when given), texture id (0-based in the
// reference, 1-based in dr_material), tiling and offset.
void channel(dr_material &m, int k, const ColoredTexture &c) {
	m.texture[k] = (c.textureId >= 0) ? c.textureId + 1 : 0;
	m.tiling[k][0] = c.tiling.x;
	m.tiling[k][1] = c.tiling.y;
	m.offset[k][0] = c.offset.x;
	m.offset[k][1] = c.offset.y;
}

// Constructor arguments of a reference material from its stored state.  DumbBasedShader stores
// its diffuse colour scaled by (1 - metal) and the library scales again, so the colour is divided
// back (exact for metal 0; a metal of 1 has no diffuse term).
bool convert_material(const Material<BakedTriFace> &src, dr_material &m, std::string &error) {
	std::memset(&m, 0, sizeof(m));
	if (holds<DumbBasedShader>(src)) {
		const DumbBasedShader &s = *src.getObject<DumbBasedShader>();
		const ColoredTexture &f = field<DbFresnel>(s), &d = field<DbDiffuse>(s);
		const ColoredTexture &nrm = field<DbNormal>(s), &cut = field<DbAlpha>(s);
		const float metal = field<DbMetal>(s);
		const float keep = 1.0f - metal;
		m.type = DR_MAT_DUMB_BASED;
		set3(m.fresnel, f.color.r, f.color.g, f.color.b);
		if (keep > 0.0f) set3(m.color, d.color.r / keep, d.color.g / keep, d.color.b / keep);
		m.specular = field<DbSpec>(s);
		m.metal = metal;
		channel(m, DR_TEX_COLOR, d);
		channel(m, DR_TEX_FRESNEL, f);
		channel(m, DR_TEX_NORMAL, nrm);
		channel(m, DR_TEX_ALPHA, cut);
		set3(m.normal_color, nrm.color.r, nrm.color.g, nrm.color.b);
		m.alpha_threshold = field<DbAlphaThreshold>(s);
	} else if (holds<SimpleStochasticShader>(src)) {
		const SimpleStochasticShader &s = *src.getObject<SimpleStochasticShader>();
		const ColorRGB &a = field<SsAlbedo>(s);
		m.type = DR_MAT_SIMPLE_STOCHASTIC;
		set3(m.color, a.r, a.g, a.b);
		m.diffuse = field<SsDiffuse>(s);
		m.smoothness = field<SsGloss>(s);
		m.shininess = field<SsShine>(s);
	} else if (holds<Shaders::FresnelShader>(src)) {
		const ColoredTexture &c = field<FrColor>(*src.getObject<Shaders::FresnelShader>());
		m.type = DR_MAT_FRESNEL;
		set3(m.color, c.color.r, c.color.g, c.color.b);
		channel(m, DR_TEX_COLOR, c);
	} else if (holds<DefaultShader>(src)) {
		const DefaultShader &s = *src.getObject<DefaultShader>();
		const ColorRGB &a = field<DfAlbedo>(s);
		m.type = DR_MAT_DEFAULT;
		set3(m.color, a.r, a.g, a.b);
		m.diffuse = field<DfDiffuse>(s);
		m.smoothness = field<DfGloss>(s);
		m.shininess = field<DfShine>(s);
	} else {
		error = "GB300Renderer: a material's shader has no counterpart in the library";
		return false;
	}
	return true;
}

// Constructor arguments of a reference light from its stored state.  The Spotlight stores cosines
// of its half-angles and its colour times the luminosity; they go back as angles (acos, within a
// few ulps) and luminosity 1.
bool convert_light(const Light &src, dr_light &l, std::string &error) {
	std::memset(&l, 0, sizeof(l));
	if (holds<SphericalLightEmitter>(src)) {
		const SphericalLightEmitter &s = *src.getObject<SphericalLightEmitter>();
		l.type = DR_LIGHT_SPHERICAL;
		set3(l.color, s.col.r, s.col.g, s.col.b);
		set3(l.position, s.pos.x, s.pos.y, s.pos.z);
		l.radius = s.rad;
	} else if (holds<SimpleSoftDirectionalLight>(src)) {
		const SimpleSoftDirectionalLight &s = *src.getObject<SimpleSoftDirectionalLight>();
		l.type = DR_LIGHT_SOFT_DIRECTIONAL;
		set3(l.color, s.color.r, s.color.g, s.color.b);
		set3(l.direction, s.dir.x, s.dir.y, s.dir.z);
		l.distance = s.dist;
		l.softness = (s.dist != 0.0f) ? s.soft / s.dist : 0.0f;   // the constructor stores distance x softness
	} else if (holds<SimpleDirectionalLight>(src, Color(1.0f, 1.0f, 1.0f), Vector3(0.0f, -1.0f, 0.0f), 1.0f)) {
		const SimpleDirectionalLight &s = *src.getObject<SimpleDirectionalLight>();
		l.type = DR_LIGHT_DIRECTIONAL;
		set3(l.color, s.color.r, s.color.g, s.color.b);
		set3(l.direction, s.dir.x, s.dir.y, s.dir.z);
		l.distance = s.dist;
	} else if (holds<Lights::Spotlight>(src)) {
		const Lights::Spotlight &s = *src.getObject<Lights::Spotlight>();
		const Color &c = field<SpColor>(s);
		const Vertex &p = field<SpPosition>(s);
		const Vector3 &d = field<SpDirection>(s);
		const uint8_t flags = field<SpFlags>(s);
		l.type = DR_LIGHT_SPOTLIGHT;
		set3(l.color, c.r, c.g, c.b);
		l.luminosity = 1.0f;
		set3(l.position, p.x, p.y, p.z);
		set3(l.direction, d.x, d.y, d.z);
		l.hotspot_angle = std::acos(std::fmax(-1.0f, std::fmin(1.0f, field<SpInner>(s)))) * kRadian;
		l.falloff_angle = std::acos(std::fmax(-1.0f, std::fmin(1.0f, field<SpOuter>(s)))) * kRadian;
		l.falloff_power = field<SpFalloff>(s);
		l.emitter_size = field<SpEmitter>(s);
		l.samples = flags & 31;
		l.cast_shadows = (flags & 32) ? 1 : 0;
		l.emit_from_sphere = (flags & 64) ? 1 : 0;
	} else {
		error = "GB300Renderer: a light has no counterpart in the library";
		return false;
	}
	return true;
}

// The device pixels of a frame buffer's device replica: FrameBuffer::getDeviceObject (a copy of
// the device handle, FrameBuffer.impl.cuh:200-216) gives the device BlockBasedFrameBuffer, and the
// registry BlockBasedFrameBuffer keeps for its device mirrors (BlockBasedFrameBuffer.impl.cuh:
// 175-201, 248-279) gives its pixel array.
float *device_pixels(const FrameBuffer *device, cudaStream_t &stream) {
	void *object = FrameBuffer::getDeviceObject(device, &stream);
	if (object == NULL) return NULL;
	std::lock_guard<std::mutex> guard(*Member<BbLock>::ptr);
	const MirrorMap &mirrors = *Member<BbMirrors>::ptr;
	MirrorMap::const_iterator it = mirrors.find(object);
	if (it == mirrors.end()) return NULL;
	return reinterpret_cast<float *>(it->second.*Member<BbData>::ptr);
}

}  // namespace

GB300Renderer::GB300Renderer(
	const ThreadConfiguration &configuration, const BlockConfiguration &blockSettings, FrameBufferManager *buffer,
	SceneType *sceneManager, CameraManager *camera, BoxingMode boxingMode, int maxBounces, int samplesPerPixelX,
	int samplesPerPixelY, int pixelsPerGPUThread, bool ignoreBackfaces)
	: DumbRenderer(configuration, blockSettings, buffer, sceneManager, camera, boxingMode, maxBounces,
		samplesPerPixelX, samplesPerPixelY, pixelsPerGPUThread, ignoreBackfaces),
	scene(NULL), converted(NULL), seed(0), tightOctree(false) {}

GB300Renderer::~GB300Renderer() {
	killRenderThreads();   // no worker thread may still be inside renderBlocksGPU
	for (size_t i = 0; i < renderers.size(); i++) dr_renderer_destroy(renderers[i]);
	if (scene != NULL) dr_scene_destroy(scene);
}

void GB300Renderer::setSeed(uint32_t value) { seed = value; }

std::string GB300Renderer::lastError() {
	std::lock_guard<std::mutex> guard(sceneLock);
	return error;
}

void GB300Renderer::invalidateScene() {
	std::lock_guard<std::mutex> guard(sceneLock);
	converted = NULL;
}

void GB300Renderer::setTightOctree(bool tight) {
	std::lock_guard<std::mutex> guard(sceneLock);
	if (tight != tightOctree) converted = NULL;
	tightOctree = tight;
}

void GB300Renderer::fail(const std::string &message) {
	std::lock_guard<std::mutex> guard(sceneLock);
	error = message;
}

bool GB300Renderer::ensureScene(std::string &err) {
	const SceneType *src = getScene();
	if (src == NULL) { err = "GB300Renderer: no scene"; return false; }
	if (scene != NULL && converted == src) return true;
	SceneType *s = const_cast<SceneType *>(src);
	const Stacktor<Renderable<BakedTriFace> > &data = s->geometry.cpuHandle()->getData();
	const int n = data.size();
	std::vector<float> xyz(9 * (size_t)n), nrm(9 * (size_t)n), uv(6 * (size_t)n);
	std::vector<int32_t> mat(n);
	for (int i = 0; i < n; i++) {
		const BakedTriFace &f = data[i].object;
		const Vertex *v[3] = {&f.vert.a, &f.vert.b, &f.vert.c};
		const Vertex *w[3] = {&f.norm.a, &f.norm.b, &f.norm.c};
		const Vertex *t[3] = {&f.tex.a, &f.tex.b, &f.tex.c};
		for (int k = 0; k < 3; k++) {
			set3(&xyz[9 * (size_t)i + 3 * k], v[k]->x, v[k]->y, v[k]->z);
			set3(&nrm[9 * (size_t)i + 3 * k], w[k]->x, w[k]->y, w[k]->z);
			uv[6 * (size_t)i + 2 * k] = t[k]->x;
			uv[6 * (size_t)i + 2 * k + 1] = t[k]->y;
		}
		mat[i] = data[i].materialId;
	}
	const Stacktor<Material<BakedTriFace> > &materials = *s->materials.cpuHandle();
	std::vector<dr_material> mats(materials.size());
	for (int i = 0; i < materials.size(); i++)
		if (!convert_material(materials[i], mats[i], err)) return false;
	const Stacktor<Light> &lights = *s->lights.cpuHandle();
	std::vector<dr_light> lts(lights.size());
	for (int i = 0; i < lights.size(); i++)
		if (!convert_light(lights[i], lts[i], err)) return false;
	dr_build_params bp;
	std::memset(&bp, 0, sizeof(bp));
	bp.device_build = 1;   // the reference's split rule, built on this worker's GPU
	bp.box_epsilon = tightOctree ? -1.0f : 0.0f;   // 0: the reference's padding; < 0: the physical-mode one
	dr_scene *out = NULL;
	if (dr_scene_create(xyz.data(), nrm.data(), mat.data(), n, mats.data(), (int32_t)mats.size(), lts.data(),
	                    (int32_t)lts.size(), &bp, &out) != DR_OK) {
		err = std::string("GB300Renderer: dr_scene_create: ") + dr_last_error();
		return false;
	}
	const Stacktor<Texture> &textures = *s->textures.cpuHandle();
	if (textures.size() > 0) {
		std::vector<std::vector<float> > texels(textures.size());
		std::vector<dr_texture> tex(textures.size());
		for (int k = 0; k < textures.size(); k++) {
			const Texture &t = textures[k];
			const uint32_t w = t.width(), h = t.height();
			texels[k].resize(4 * (size_t)w * h);
			for (uint32_t y = 0; y < h; y++)
				for (uint32_t x = 0; x < w; x++) {
					const Color &c = t(x, y);
					float *p = &texels[k][4 * ((size_t)y * w + x)];
					p[0] = c.r; p[1] = c.g; p[2] = c.b; p[3] = c.a;
				}
			tex[k].width = (int32_t)w;
			tex[k].height = (int32_t)h;
			tex[k].filtering = (t.filtering() == Texture::FILTER_BILINEAR) ? DR_FILTER_BILINEAR : DR_FILTER_NONE;
			tex[k].rgba = texels[k].data();
		}
		if (dr_scene_set_textures(out, tex.data(), (int32_t)tex.size(), uv.data()) != DR_OK) {
			err = std::string("GB300Renderer: dr_scene_set_textures: ") + dr_last_error();
			dr_scene_destroy(out);
			return false;
		}
	}
	if (scene != NULL) dr_scene_destroy(scene);
	scene = out;
	converted = src;
	return true;
}

bool GB300Renderer::threadRenderer(int slot, dr_renderer **out, std::string &err) {
	std::lock_guard<std::mutex> guard(sceneLock);
	if (slot < 0) { err = "GB300Renderer: bad thread slot"; return false; }
	if ((size_t)slot >= renderers.size()) renderers.resize((size_t)slot + 1, NULL);
	if (renderers[slot] == NULL && dr_renderer_create(0, &renderers[slot]) != DR_OK) {
		err = std::string("GB300Renderer: dr_renderer_create: ") + dr_last_error();
		return false;
	}
	*out = renderers[slot];
	return true;
}

bool GB300Renderer::toCamera(dr_camera &c, std::string &err) {
	CameraManager *manager = getCamera();
	const Camera *cam = (manager != NULL) ? manager->cpuHandle() : NULL;
	if (cam == NULL || cam->lense.object() == NULL) { err = "GB300Renderer: no camera / lens"; return false; }
	std::memset(&c, 0, sizeof(c));
	const Lense &lens = cam->lense;
	if (holds<SimpleStochasticLense>(lens)) {
		c.lens = DR_LENS_SIMPLE_STOCHASTIC;
		c.lens_x = field<StochX>(*lens.getObject<SimpleStochasticLense>());
	} else if (holds<DefaultPerspectiveLense>(lens)) {
		c.lens = DR_LENS_DEFAULT_PERSPECTIVE;
		c.lens_x = field<PerspX>(*lens.getObject<DefaultPerspectiveLense>());
	} else if (holds<Lenses::SphericalSegmentLense>(lens)) {
		const Lenses::SphericalSegmentLense &s = *lens.getObject<Lenses::SphericalSegmentLense>();
		const Vector2 &a = field<SegAlpha>(s);
		const Color &f = field<SegFilter>(s);
		c.lens = DR_LENS_SPHERICAL_SEGMENT;
		c.angle[0] = a.x;
		c.angle[1] = a.y;
		c.focal_distance = field<SegDist>(s);
		c.softness = field<SegSoft>(s);
		set3(c.filter, f.r, f.g, f.b);
	} else {
		err = "GB300Renderer: the camera's lens has no counterpart in the library";
		return false;
	}
	if (c.lens_x > 0.0f) c.angle[0] = c.angle[1] = 2.0f * std::atan(0.5f / c.lens_x) * kRadian;   // informational
	// directions: Transform::direction's basis; origins: the point transform's rows (Camera.impl.cuh:7-10)
	const Transform &t = cam->transform;
	const Vector3 r = t.right(), u = t.up(), fw = t.front();
	set3(c.right, r.x, r.y, r.z);
	set3(c.up, u.x, u.y, u.z);
	set3(c.forward, fw.x, fw.y, fw.z);
	Transform z = t;
	z.setPosition(Vector3(0.0f, 0.0f, 0.0f));
	const Vector3 cx = Vector3(1.0f, 0.0f, 0.0f) >> z, cy = Vector3(0.0f, 1.0f, 0.0f) >> z, cz = Vector3(0.0f, 0.0f, 1.0f) >> z;
	set3(c.row_x, cx.x, cy.x, cz.x);
	set3(c.row_y, cx.y, cy.y, cz.y);
	set3(c.row_z, cx.z, cy.z, cz.z);
	const Vector3 &p = t.getPosition();
	set3(c.position, p.x, p.y, p.z);
	c.origin_rows = 1;
	return true;
}

bool GB300Renderer::renderDeviceBlocks(int threadSlot, float *deviceBlocks, int width, int height, int startBlock,
                                       int endBlock, cudaStream_t stream) {
	std::string err;
	{
		std::lock_guard<std::mutex> guard(sceneLock);
		if (!ensureScene(err)) { error = err; return false; }
	}
	dr_renderer *r = NULL;
	if (!threadRenderer(threadSlot, &r, err)) { fail(err); return false; }
	dr_camera cam;
	if (!toCamera(cam, err)) { fail(err); return false; }
	dr_render_params p;
	std::memset(&p, 0, sizeof(p));
	p.mode = DR_MODE_REFERENCE;
	p.width = width;
	p.height = height;
	p.samples_x = getSamplesPerPixelX();
	p.samples_y = getSamplesPerPixelY();
	p.max_bounces = getMaxBounces();
	p.cull_backfaces = getIgnoreBackfaces() ? 1 : 0;
	p.boxing = (int32_t)getBoxingMode();
	p.iteration = (int32_t)iteration();
	p.seed = seed;
	if (dr_render_blocks(r, scene, &cam, deviceBlocks, startBlock, endBlock, &p, stream) != DR_OK) {
		fail(std::string("GB300Renderer: dr_render_blocks: ") + dr_last_error());
		return false;
	}
	// as the reference renderer does, the call returns once its blocks are written
	const cudaError_t e = cudaStreamSynchronize(stream);
	if (e != cudaSuccess) {
		fail(std::string("GB300Renderer: stream: ") + cudaGetErrorString(e));
		return false;
	}
	return true;
}

bool GB300Renderer::renderBlocksGPU(const Info &info, FrameBuffer *host, FrameBuffer *device, int startBlock,
                                    int endBlock, cudaStream_t &renderStream) {
	int width = 0, height = 0;
	host->getSize(&width, &height);
	// the library writes BlockBasedFrameBuffer<8, 16> block-major pixels: check that layout
	int bx = -1, by = -1;
	if (host->getBlockSize() != DR_BLOCK_W * DR_BLOCK_H || !host->blockPixelLocation(0, DR_BLOCK_W, &bx, &by) ||
	    bx != 0 || by != 1) {
		fail("GB300Renderer: the frame buffer is not an 8x16 block-major BlockBasedFrameBuffer");
		return false;
	}
	float *pixels = device_pixels(device, renderStream);
	if (pixels == NULL) {
		fail("GB300Renderer: the device frame buffer's pixels are not registered");
		return false;
	}
	return renderDeviceBlocks(info.globalThreadId, pixels, width, height, startBlock, endBlock, renderStream);
}
