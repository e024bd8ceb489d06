// dr_shading.cuh - device shading models.
//
// Reference semantics (DR_MODE_REFERENCE): DumbBasedShader, SimpleStochasticShader, FresnelShader and
// DefaultShader (__source__/DataStructures/Objects/Components/Shaders/DumbBasedShader/DumbBasedShader.impl.cuh:18-122,
//  .../SimpleStochasticShader/SimpleStochasticShader.impl.cuh:13-37, .../FresnelShader/FresnelShader.impl.cuh:11-19,
//  .../DefaultShader/DefaultShader.impl.cuh:3-52), the four lights (.../Scene/Lights/*:
//  SphericalLightEmitter.impl.cuh:10-18, SimpleSoftDirectionalLight.impl.cuh:12-19,
//  SimpleDirectionalLight.impl.cuh:13-16, Spotlight.impl.cuh:35-77) and lenses (.../Components/Lenses/*).  getReflectedColor is
// linear in the photon colour, so every function here returns the colour FACTOR and callers multiply.
// Physical semantics (DR_MODE_PHYSICAL): Lambert / mirror / GGX glossy with emissive triangles.
#pragma once
#include "../../include/dr_api.h"
#include "dr_device.cuh"

namespace drd {

struct c3 {
    float r, g, b;
};
__device__ __forceinline__ c3 mkc(float r, float g, float b) { return c3{r, g, b}; }
__device__ __forceinline__ c3 cmul(c3 a, c3 b) { return c3{a.r * b.r, a.g * b.g, a.b * b.b}; }
__device__ __forceinline__ c3 cscale(c3 a, float f) { return c3{a.r * f, a.g * f, a.b * f}; }
__device__ __forceinline__ c3 cadd(c3 a, c3 b) { return c3{a.r + b.r, a.g + b.g, a.b + b.b}; }

// plain float3 helpers (shading only; contraction is disabled for the whole library)
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 mul3(f3 a, float f) { return f3{a.x * f, a.y * f, a.z * f}; }
__device__ __forceinline__ f3 neg3(f3 a) { return f3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 v) { return f3{a.y * v.z - v.y * a.z, v.x * a.z - a.x * v.z, a.x * v.y - v.x * a.y}; }
__device__ __forceinline__ float sqr3(f3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ f3 norm3(f3 a) { float im = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); return f3{a.x * im, a.y * im, a.z * im}; }
__device__ __forceinline__ f3 divf3(f3 a, float f) { float fi = 1.0f / f; return f3{a.x * fi, a.y * fi, a.z * fi}; }
__device__ __forceinline__ f3 reflect3(f3 v, f3 n) { float m = (2.0f * dot3(v, n) / sqr3(n)); return f3{v.x - n.x * m, v.y - n.y * m, v.z - n.z * m}; }
__device__ __forceinline__ f3 normal_on3(f3 a, f3 v) { return mul3(v, dot3(a, v) / sqr3(v)); }

struct TriV {
    f3 a, b, c;
};
__device__ __forceinline__ TriV load_tri(const float4 *p, int i) {
    float4 A = __ldg(p + 3 * (size_t)i), B = __ldg(p + 3 * (size_t)i + 1), C = __ldg(p + 3 * (size_t)i + 2);
    return TriV{f3of(A), f3of(B), f3of(C)};
}
// Triangle::normal() = (c - a) x (b - a)
__device__ __forceinline__ f3 tri_normal(const TriV &t) { return cross3(sub3(t.c, t.a), sub3(t.b, t.a)); }

// Triangle::getMasses (Triangle.impl.h:248-276)
__device__ inline f3 get_masses(const TriV &t, f3 center) {
    f3 ab = sub3(t.b, t.a);
    f3 bc = sub3(t.c, t.b);
    f3 ae = sub3(ab, normal_on3(ab, bc));
    f3 ax = sub3(center, t.a);
    f3 ad = normal_on3(ax, ae);
    if (ae.x < 0) { ad.x = -ad.x; ae.x = -ae.x; }
    if (ae.y < 0) { ad.y = -ad.y; ae.y = -ae.y; }
    if (ae.z < 0) { ad.z = -ad.z; ae.z = -ae.z; }
    float div = ad.x + ad.y + ad.z;
    if (div == 0) return f3{1, 0, 0};
    float g = (ae.x + ae.y + ae.z) / div;
    float tt;
    f3 by = sub3(add3(t.a, mul3(ax, g)), t.b);
    if (bc.x < 0) { bc.x = -bc.x; by.x = -by.x; }
    if (bc.y < 0) { bc.y = -bc.y; by.y = -by.y; }
    if (bc.z < 0) { bc.z = -bc.z; by.z = -by.z; }
    div = bc.x + bc.y + bc.z;
    tt = (div == 0) ? 0.0f : (by.x + by.y + by.z) / div;
    float cc = tt, bb = (1 - tt), aa = (g - 1);
    return divf3(f3{aa, bb, cc}, aa + bb + cc);
}
__device__ __forceinline__ f3 mass_center(const TriV &t, f3 m) { return add3(add3(mul3(t.a, m.x), mul3(t.b, m.y)), mul3(t.c, m.z)); }

// DumbRand::pointOnSphere from two uniforms (DumbRand.impl.cuh:70-77)
__device__ __forceinline__ f3 point_on_sphere(float u0, float u1, float radius) {
    float theta = (2.0f * 3.14159265359f * u0);
    float cosPhi = (1.0f - (2.0f * u1));
    float sinPhi = sqrtf(1.0f - (cosPhi * cosPhi));
    return f3{(sinPhi * cosf(theta)) * radius, (sinPhi * sinf(theta)) * radius, cosPhi * radius};
}

// ---- textures (Texture.impl.cuh:81-95; ColoredTexture, DumbStructs.cuh:88-131) ------------------
__device__ __forceinline__ float4 texel(const Scene &S, int4 info, uint32_t x, uint32_t y) {
    return __ldg(S.texels + info.x + (size_t)y * (uint32_t)info.y + x);
}
__device__ __forceinline__ float4 f4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4mul(float4 a, float f) { return make_float4(a.x * f, a.y * f, a.z * f, a.w * f); }
// Texture::operator()(Vector2): u, v wrapped into [0, 1), v flipped, nearest or bilinear texel(s).
__device__ inline float4 tex_lookup(const Scene &S, int t, float u, float v) {
    const int4 info = __ldg(S.tex_info + t);
    const uint32_t w = (uint32_t)info.y, h = (uint32_t)info.z;
    float x = (u + ((float)(((int)(-u)) + 2)));
    x -= ((float)((int)x));
    float y = (v + ((float)(((int)(-v)) + 2)));
    y -= ((float)((int)y));
    y = (1.0f - y);
    const float px = (x * ((float)w)), py = (y * ((float)h));
    const uint32_t min_x = (((uint32_t)px) % w), min_y = (((uint32_t)py) % h);
    const uint32_t max_x = ((min_x + 1) % w), max_y = ((min_y + 1) % h);
    const float off_x = (px - ((float)min_x)), off_y = (py - ((float)min_y));
    if (info.w == DR_FILTER_NONE) return texel(S, info, (off_x <= 0.5f) ? min_x : max_x, (off_y <= 0.5f) ? min_y : max_y);
    return f4add(f4add(f4add(f4mul(texel(S, info, min_x, min_y), ((1.0f - off_x) * (1.0f - off_y))),
                             f4mul(texel(S, info, min_x, max_y), ((1.0f - off_x) * off_y))),
                       f4mul(texel(S, info, max_x, min_y), (off_x * (1.0f - off_y)))),
                 f4mul(texel(S, info, max_x, max_y), (off_x * off_y)));
}
// Texture coordinate of a hit: the corner coordinates weighted by the hit's masses (tex.massCenter).
__device__ __forceinline__ float2 hit_uv(const Scene &S, int tri, f3 m) {
    const float2 a = __ldg(S.uv + 3 * (size_t)tri), b = __ldg(S.uv + 3 * (size_t)tri + 1), c = __ldg(S.uv + 3 * (size_t)tri + 2);
    return make_float2(((a.x * m.x) + (b.x * m.y)) + (c.x * m.z), ((a.y * m.x) + (b.y * m.y)) + (c.y * m.z));
}
// The texel a material channel reads at `uv`: texture(uv x tiling + offset).
__device__ __forceinline__ float4 channel_texel(const Scene &S, const Material &m, int ch, float2 uv) {
    return tex_lookup(S, m.texture[ch], (uv.x * m.tiling[ch][0]) + m.offset[ch][0], (uv.y * m.tiling[ch][1]) + m.offset[ch][1]);
}
__device__ __forceinline__ bool any_texture(const Material &m) {
    return m.texture[0] >= 0 || m.texture[1] >= 0 || m.texture[2] >= 0 || m.texture[3] >= 0;
}
// Alpha cutout: the surface lets paths through where alpha_threshold >= alpha (colour alpha 1).
__device__ __forceinline__ bool cut_out(const Scene &S, const Material &m, float2 uv) {
    return m.texture[DR_TEX_ALPHA] >= 0 && m.alpha_threshold >= (1.0f * channel_texel(S, m, DR_TEX_ALPHA, uv).w);
}
// Shading normal: the interpolated normal, or with a normal map (ColoredTexture::getNormal) the
// mapped normal in the frame of that normal, a tangent from the corner texture coordinates and
// their cross product.
__device__ inline f3 shading_normal(const Scene &S, const Material &m, int tri, const TriV &v, const TriV &nt, f3 masses, float2 uv) {
    f3 n = norm3(mass_center(nt, masses));
    if (m.texture[DR_TEX_NORMAL] < 0) return n;
    float2 td;
    f3 vd;
    const f3 mc = mass_center(v, masses);
    if (masses.x < 0.999f) {
        const float2 a = __ldg(S.uv + 3 * (size_t)tri);
        td = make_float2(a.x - uv.x, a.y - uv.y);
        vd = sub3(v.a, mc);
    } else {
        const float2 b = __ldg(S.uv + 3 * (size_t)tri + 1);
        td = make_float2(b.x - uv.x, b.y - uv.y);
        vd = sub3(v.b, mc);
    }
    const f3 co = norm3(cross3(vd, n));
    vd = cross3(co, n);
    const f3 u = norm3(sub3(mul3(vd, td.y), mul3(co, td.x)));
    const f3 w = cross3(u, n);
    const float4 rgb = channel_texel(S, m, DR_TEX_NORMAL, uv);
    const f3 k = f3{m.normal_color[1] * rgb.z, m.normal_color[0] * ((rgb.x * 2.0f) - 1.0f), m.normal_color[2] * ((rgb.y * 2.0f) - 1.0f)};
    return norm3(add3(add3(mul3(n, k.x), mul3(u, k.y)), mul3(w, k.z)));
}

// ---- DumbBasedShader -------------------------------------------------------------------------
__device__ inline bool dumb_based_request(const Scene &S, int tri, const Material &m, const TriV &v, const TriV &nt, f3 hit,
                                          f3 raydir, uint32_t key, uint32_t bounce, f3 &dir, int &type) {
    f3 normal = norm3(tri_normal(v));
    f3 masses = get_masses(v, hit);
    const bool textured = any_texture(m);
    const float2 uv = textured ? hit_uv(S, tri, masses) : make_float2(0.0f, 0.0f);
    if (textured && cut_out(S, m, uv)) {
        dir = raydir;
        type = 3;
        return true;
    }
    float metal = fmaxf(fminf(m.metal, 1.0f), 0.0f);
    if (rnd(key, bounce, 0) <= metal) {
        f3 n = shading_normal(S, m, tri, v, nt, masses, uv);
        if (dot3(n, raydir) >= 0.0f) return false;
        f3 r = norm3(reflect3(raydir, n));
        if (dot3(r, normal) < 0) normal = mul3(normal, -1.0f);
        f3 a = cross3(r, f3{1.0f, 0.0f, 0.0f});
        if (sqr3(normal) < kEps) a = cross3(r, f3{0.0f, 1.0f, 0.0f});
        a = norm3(a);
        f3 b = cross3(r, a);
        f3 sd = f3{0, 0, 0};
        for (int tries = 0; tries < 32; tries++) {
            float cosine = powf(rnd(key, bounce, 8 + 2 * tries), 1.0f / m.specular);
            float sinus = sqrtf(1.0f - (cosine * cosine));
            float angle = (rnd(key, bounce, 9 + 2 * tries) * 2.0f * 3.14159265359f);
            float angleCos = cosf(angle);
            float angleSin = sqrtf(1.0f - (angleCos * angleCos));
            sd = add3(mul3(r, cosine), mul3(add3(mul3(a, angleCos), mul3(b, angleSin)), sinus));
            if (dot3(sd, normal) >= 0.0f) break;
        }
        dir = sd;
        type = 1;
        return true;
    }
    f3 sd = point_on_sphere(rnd(key, bounce, 1), rnd(key, bounce, 2), 1.0f);
    if (dot3(sd, normal) < 0.0f) sd = mul3(sd, -1.0f);
    dir = sd;
    type = 2;
    return true;
}

__device__ inline c3 dumb_based_reflect(const Scene &S, int tri, const Material &m, const TriV &v, const TriV &nt, f3 hit,
                                        f3 photon_dir, f3 observer, bool direct, int sample_type) {
    f3 masses = get_masses(v, hit);
    const bool textured = any_texture(m);
    const float2 uv = textured ? hit_uv(S, tri, masses) : make_float2(0.0f, 0.0f);
    if (textured && cut_out(S, m, uv)) {
        const float pass = (dot3(norm3(observer), norm3(photon_dir)) >= 0.9999f) ? 1.0f : 0.0f;
        return mkc(pass, pass, pass);
    }
    if (dot3(norm3(tri_normal(v)), photon_dir) > 0.0f)
        if (!direct) return mkc(1, 1, 1);
    if (dot3(mass_center(nt, masses), observer) < 0.0f) return mkc(0, 0, 0);
    f3 n = shading_normal(S, m, tri, v, nt, masses, uv);
    f3 wi = neg3(norm3(photon_dir));
    float metal = fmaxf(fminf(m.metal, 1.0f), 0.0f);
    float spec = m.specular;
    c3 brdf = mkc(0, 0, 0);
    bool brdfMatters = (direct || sample_type == 1);
    if (brdfMatters) {
        f3 w0 = norm3(observer);
        f3 wh = norm3(add3(w0, wi));
        float val = (1.0f - dot3(wh, wi));
        float sq = val * val;
        float f5 = sq * sq * val;
        c3 fres = mkc(m.fresnel[0], m.fresnel[1], m.fresnel[2]);
        if (m.texture[DR_TEX_FRESNEL] >= 0) {
            const float4 t = channel_texel(S, m, DR_TEX_FRESNEL, uv);
            fres = mkc(fres.r * t.x, fres.g * t.y, fres.b * t.z);
        }
        c3 fwi = mkc(fres.r + (1 - fres.r) * f5, fres.g + (1 - fres.g) * f5, fres.b + (1 - fres.b) * f5);
        float multiplier;
        if (direct) {
            float dwh = ((spec + 2) / (2.0f * 3.14159265359f)) * powf(dot3(n, wh), spec);
            float gwiw0 = fminf(1.0f, fminf(2.0f * dot3(n, wh) * dot3(n, w0) / dot3(w0, wh),
                                            2.0f * dot3(n, wh) * dot3(n, wi) / dot3(w0, wh)));
            multiplier = (dwh * gwiw0) / (4.0f * dot3(n, w0) * dot3(n, wi));
        } else multiplier = 1.0f;
        c3 bb = cscale(fwi, multiplier);
        brdf = mkc(fmaxf(0.0f, fminf(bb.r, 1.0f)), fmaxf(0.0f, fminf(bb.g, 1.0f)), fmaxf(0.0f, fminf(bb.b, 1.0f)));
    }
    bool diffuseMatters = (direct || sample_type == 2);
    c3 diff = cscale(mkc(m.color[0], m.color[1], m.color[2]), 1.0f - metal);
    if (m.texture[DR_TEX_COLOR] >= 0) {
        const float4 t = channel_texel(S, m, DR_TEX_COLOR, uv);
        diff = mkc(diff.r * t.x, diff.g * t.y, diff.b * t.z);
    }
    c3 diffuse = diffuseMatters ? cscale(diff, dot3(n, wi)) : mkc(0, 0, 0);
    if (brdfMatters && diffuseMatters)
        return mkc(fmaxf(0.0f, fminf((brdf.r * metal) + diffuse.r, 1.0f)), fmaxf(0.0f, fminf((brdf.g * metal) + diffuse.g, 1.0f)),
                   fmaxf(0.0f, fminf((brdf.b * metal) + diffuse.b, 1.0f)));
    if (brdfMatters) return brdf;
    return cscale(diffuse, 1.0f / (1.0f - metal));
}

// ---- SimpleStochasticShader ------------------------------------------------------------------
__device__ __forceinline__ void ss_params(const Material &m, float &diff, float &gloss) {
    float total = m.diffuse + m.smoothness;
    float mul = ((total > 1.0f) ? (1.0f / total) : 1.0f);
    diff = m.diffuse * mul;
    gloss = m.smoothness * mul;
}
__device__ inline f3 ss_request(const Material &m, const TriV &v, const TriV &nt, f3 hit, f3 raydir, uint32_t key, uint32_t bounce) {
    float diff, gloss;
    ss_params(m, diff, gloss);
    f3 direction = point_on_sphere(rnd(key, bounce, 1), rnd(key, bounce, 2), 1.0f);
    if (dot3(direction, tri_normal(v)) < 0) direction = neg3(direction);
    f3 hn = mass_center(nt, get_masses(v, hit));
    f3 refl = reflect3(raydir, hn);
    return norm3(add3(mul3(direction, diff), mul3(refl, gloss)));
}
__device__ inline c3 ss_reflect(const Material &m, const TriV &v, const TriV &nt, f3 hit, f3 photon_dir, f3 observer) {
    float diff, gloss;
    ss_params(m, diff, gloss);
    f3 hn = mass_center(nt, get_masses(v, hit));
    f3 refl = reflect3(photon_dir, hn);
    float rc = dot3(refl, hn) / sqrtf(sqr3(refl) * sqr3(hn));
    if (rc < 0.0f) rc = 0.0f;
    float oc = dot3(observer, refl) / sqrtf(sqr3(observer) * sqr3(refl));
    if (oc < 0.0f) oc = 0.0f;
    return cscale(mkc(m.color[0], m.color[1], m.color[2]), (diff * rc) + (gloss * powf(oc, m.shininess)));
}

// ---- FresnelShader: no indirect samples; DumbTools::fresnel(colour, interpolated normal, -photon
// direction) (FresnelShader.impl.cuh:11-19, DumbStructs.cuh:136-140); the normal is not normalised.
__device__ inline c3 fresnel_reflect(const Scene &S, int tri, const Material &m, const TriV &v, const TriV &nt, f3 hit,
                                     f3 photon_dir) {
    f3 masses = get_masses(v, hit);
    f3 light = neg3(norm3(photon_dir));
    f3 normal = mass_center(nt, masses);
    c3 col = mkc(m.color[0], m.color[1], m.color[2]);
    if (m.texture[DR_TEX_COLOR] >= 0) {
        const float4 t = channel_texel(S, m, DR_TEX_COLOR, hit_uv(S, tri, masses));
        col = mkc(col.r * t.x, col.g * t.y, col.b * t.z);
    }
    float val = (1.0f - dot3(normal, light));
    float sq = (val * val);
    float f = sq * sq * val;
    return mkc(col.r + ((1.0f - col.r) * f), col.g + ((1.0f - col.g) * f), col.b + ((1.0f - col.b) * f));
}

// ---- DefaultShaderGeneric (DefaultShader.impl.cuh:3-52): one sample along the reflection of the
// ray about the interpolated normal (not normalised, weight 1, type 0); reflected colour
// albedo x (diff cosL + gloss max(cos(refl, observer), 0)^shininess) with the constructor's
// diffuse / smoothness normalisation; the observer is (hit + direction) - hit, as the reference
// forms it.
__device__ inline f3 default_request(const TriV &v, const TriV &nt, f3 hit, f3 raydir) {
    return reflect3(raydir, mass_center(nt, get_masses(v, hit)));
}
__device__ inline c3 default_reflect(const Material &m, const TriV &v, const TriV &nt, f3 hit, f3 photon_dir, f3 observer) {
    float diff, gloss;
    ss_params(m, diff, gloss);
    f3 normal = mass_center(nt, get_masses(v, hit));
    f3 cam = sub3(add3(hit, observer), hit);
    f3 refl = reflect3(photon_dir, normal);
    float cosL = fmaxf(dot3(refl, normal) / sqrtf(sqr3(refl) * sqr3(normal)), 0.0f);
    float oc = fmaxf(dot3(refl, cam) / sqrtf(sqr3(refl) * sqr3(cam)), 0.0f);
    return cscale(mkc(m.color[0], m.color[1], m.color[2]), (diff * cosL) + (gloss * powf(oc, m.shininess)));
}

// Material::getReflectedColor dispatch (colour factor).  The physical-mode types take the
// SimpleStochastic branch, as they always have in the reference mode.
__device__ inline c3 ref_reflect(const Scene &S, int tri, f3 hit, f3 photon_dir, f3 observer, bool direct, int sample_type) {
    const Material &m = S.mats[__ldg(S.mat_id + tri)];
    TriV v = load_tri(S.tris, tri), nt = load_tri(S.nrms, tri);
    if (m.type == 0) return dumb_based_reflect(S, tri, m, v, nt, hit, photon_dir, observer, direct, sample_type);
    if (m.type == DR_MAT_FRESNEL) return fresnel_reflect(S, tri, m, v, nt, hit, photon_dir);
    if (m.type == DR_MAT_DEFAULT) return default_reflect(m, v, nt, hit, photon_dir, observer);
    return ss_reflect(m, v, nt, hit, photon_dir, observer);
}

// Light::getVertexPhotons (photon origin, direction, colour) for light `li`.
__device__ inline void light_photon(const Light &l, f3 point, uint32_t key, uint32_t bounce, int li, f3 &o, f3 &d, c3 &c) {
    uint32_t d0 = 72 + 3 * (uint32_t)li;
    if (l.type == 0) {
        f3 ep = point_on_sphere(rnd(key, bounce, d0), rnd(key, bounce, d0 + 1), l.radius);
        ep = mul3(ep, rnd(key, bounce, d0 + 2));
        ep = add3(ep, f3{l.position[0], l.position[1], l.position[2]});
        f3 delta = sub3(point, ep);
        o = ep;
        d = norm3(delta);
        float inv = 1.0f / sqr3(delta);
        c = mkc(l.color[0] * inv, l.color[1] * inv, l.color[2] * inv);
    } else if (l.type == 1) {
        f3 dir = norm3(f3{l.direction[0], l.direction[1], l.direction[2]});
        float soft = l.distance * l.softness;
        float rad = soft * rnd(key, bounce, d0);
        f3 off = point_on_sphere(rnd(key, bounce, d0 + 1), rnd(key, bounce, d0 + 2), rad);
        f3 origin = add3(sub3(point, mul3(dir, l.distance)), off);
        o = origin;
        d = sub3(point, origin);
        c = mkc(l.color[0], l.color[1], l.color[2]);
    } else {
        f3 dir = norm3(f3{l.direction[0], l.direction[1], l.direction[2]});
        o = sub3(point, mul3(dir, l.distance));
        d = dir;
        c = mkc(l.color[0], l.color[1], l.color[2]);
    }
}

// Photons light `l` sends toward one shading point: a spotlight's sample count, else 1.
__device__ __forceinline__ int light_photons(const Light &l) { return (l.type == DR_LIGHT_SPOTLIGHT) ? l.samples : 1; }

// Spotlight::getVertexPhotons, photon k of `count` (Spotlight.impl.cuh:35-77): a point on the
// emitter disc (ver / hor frame about the direction) or in the emitter sphere, colour scaled by
// emitter area over emitter + spread area (the disc area is left out for a sphere) and the cubic
// falloff between the hotspot and falloff cones.  Returns false where the reference skips the
// photon (point on the emitter, outside the falloff cone).  Random dimensions 4096 + 64 li + 3 k.
__device__ inline bool spot_photon(const Light &l, f3 point, uint32_t key, uint32_t bounce, int li, int k, f3 &o, f3 &d,
                                   c3 &c) {
    const uint32_t d0 = 4096u + 64u * (uint32_t)li + 3u * (uint32_t)k;
    const f3 dir = f3{l.direction[0], l.direction[1], l.direction[2]};
    const f3 pos0 = f3{l.position[0], l.position[1], l.position[2]};
    f3 non_dir = (dir.z > 0.9f) ? f3{1.0f, 0.0f, 0.0f} : f3{0.0f, 0.0f, 1.0f};
    f3 ver = norm3(cross3(dir, non_dir));
    f3 hor = cross3(dir, ver);
    f3 pos;
    if (l.sphere) {
        pos = point_on_sphere(rnd(key, bounce, d0), rnd(key, bounce, d0 + 1), l.emitter);
        pos = mul3(pos, rnd(key, bounce, d0 + 2));
        pos = add3(pos, pos0);
    } else {
        float angle = (rnd(key, bounce, d0) * ((2.0f * 3.14159265359f) - 0.0f)) + 0.0f;
        f3 ring = add3(mul3(ver, cosf(angle)), mul3(hor, sinf(angle)));
        pos = add3(pos0, mul3(mul3(ring, l.emitter), sqrtf(rnd(key, bounce, d0 + 1))));
    }
    f3 delta = sub3(point, pos);
    float sqr_distance = sqr3(delta);
    if (sqr_distance < kEps) return false;
    float distance = sqrtf(sqr_distance);
    float base = (l.emitter * l.emitter);
    float spread = fmaxf(1.0f - l.outer_cos, kEps);
    float surface = ((l.sphere ? 0.0f : base) + (sqr_distance * spread));
    float s = (base / (((float)l.samples) * surface));
    c = mkc(l.color[0] * s, l.color[1] * s, l.color[2] * s);
    f3 dd = divf3(delta, distance);
    float cosine = dot3(dd, dir);
    if (cosine < l.inner_cos) {
        if (cosine < l.outer_cos) return false;
        float a = ((l.inner_cos - cosine) / (l.inner_cos - l.outer_cos));
        float b = (1.0f - a);
        c = cscale(c, powf((a * b * b) + (b * (1.0f - (a * a))), l.falloff));
    }
    o = pos;
    d = dd;
    return true;
}

// ---- physical mode ---------------------------------------------------------------------------
__device__ __forceinline__ void onb(f3 n, f3 &t, f3 &b) {
    float s = n.z >= 0 ? 1.0f : -1.0f;
    float a = -1.0f / (s + n.z);
    float bb = n.x * n.y * a;
    t = f3{1.0f + s * n.x * n.x * a, s * bb, -s * n.x};
    b = f3{bb, s + n.y * n.y * a, -n.y};
}
__device__ __forceinline__ float ggx_d(float ndh, float a) {
    float a2 = a * a;
    float c2 = ndh * ndh;
    float den = c2 * (a2 - 1.0f) + 1.0f;
    return a2 / (3.14159265358979f * den * den);
}
__device__ __forceinline__ float ggx_g1(float ndv, float a) {
    float a2 = a * a;
    return 2.0f * ndv / (ndv + sqrtf(a2 + (1.0f - a2) * ndv * ndv));
}
__device__ __forceinline__ float mis2(float a, float b) { return (a * a) / (a * a + b * b); }
__device__ __forceinline__ float tri_area(const TriV &t) { return 0.5f * sqrtf(sqr3(cross3(sub3(t.b, t.a), sub3(t.c, t.a)))); }

}  // namespace drd
