// dr_dumb.cpp - DumbRay scene files (.dumb): the reference's JSON dialect and scene description,
// loaded into the host arrays that dr_scene_create and the renderer take.
//
// Restates, with the reference's float arithmetic and error rules:
//  * the Dson text format (Namespaces/Dson/Dson.cu:225-447): JSON values, dictionary keys unique,
//    numbers read as the longest decimal prefix of a token (the reference streams the token into a
//    double, so trailing characters are ignored), string escapes \" \\ \/ \b \f \n \r \t;
//  * DumbRenderContext::fromFile / fromDson (DataStructures/DumbRenderContext/DumbRenderContext.cu:
//    300-372): "include", "materials", "lights", "groups", "objects", "camera", "renderer", in that
//    order, includes parsed into the same context with paths relative to the including file;
//  * materials (parseMaterial, :654-684): DumbBasedShader::fromDson (Shaders/DumbBasedShader/
//    DumbBasedShader.impl.cuh:125-179, presets :9-12 of the header, constructor :5-15),
//    SimpleStochasticShader::fromDson (SimpleStochasticShader.impl.cuh:4-12, 39-66) and
//    Shaders::FresnelShader::fromDson (FresnelShader.impl.cuh:20-24);
//  * lights: SimpleSoftDirectionalLight::fromDson (SimpleSoftDirectionalLight.impl.cuh:5-10, 25-49),
//    SphericalLightEmitter::fromDson (SphericalLightEmitter.impl.cuh:5-9, 20-41),
//    Lights::Spotlight::fromDson (Spotlight.impl.cuh:79-151);
//  * groups and objects (DumbRenderContext.cu:103-259, 738-790): items place OBJ objects through
//    their Transform, groups apply fallback / override materials and their own Transform after
//    their members', top-level objects must end up with a material;
//  * Transform::fromDson and rebake (Objects/Components/Transform/Transform.impl.h:209-281) with
//    Vector3::rotateTwoAxisAgainstThisRadian (Primitives/Pure/Vector3/Vector3.impl.h:455-512),
//    BakedTriFace >> Transform (Meshes/BakedTriMesh/BakedTriMesh.impl.h:16-18);
//  * the camera (parseCamera, :491-530; SimpleStochasticLense / SphericalSegmentLense ::fromDson)
//    and renderer settings (parseRenderer, :531-633).
//  * textures (getImageId, DumbRenderContext.cu:374-450; ColoredTexture::fromDson, DumbStructs.cu:7-37):
//    PNG files decoded by dr_png_read, named or by path, nearest or bilinear filtering; texture
//    coordinates from the OBJ files.
// Mesh primitives (left unimplemented by the reference) fail with a message.
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/dr_api.h"
#include "dr_guard.h"

void dr_internal_set_error(const char *msg);

namespace {

// ---- Dson values --------------------------------------------------------------------------------
struct JValue {
    enum Kind { NUL, BOOL, NUM, STR, ARR, DICT } kind = NUL;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> dict;

    const JValue *get(const char *key) const {
        for (const auto &kv : dict)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    bool has(const char *key) const { return get(key) != nullptr; }
};

struct LoadError {
    std::string msg;
};
[[noreturn]] void raise(const std::string &msg) { throw LoadError{msg}; }

class JParser {
  public:
    explicit JParser(const std::string &text) : s_(text) {}

    JValue parse_document() {
        skip_ws();
        if (i_ >= s_.size()) raise("empty document");
        JValue v = value();
        skip_ws();
        if (i_ < s_.size()) raise("more than one value at the top level");
        return v;
    }

  private:
    const std::string &s_;
    size_t i_ = 0;
    int depth_ = 0;  // container nesting; bounded so hostile text cannot exhaust the stack

    static bool ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }
    static bool structural(char c) { return c == '{' || c == '}' || c == '[' || c == ']' || c == ',' || c == ':' || c == '"'; }
    void skip_ws() {
        while (i_ < s_.size() && ws(s_[i_])) i_++;
    }
    [[noreturn]] void fail(const std::string &what) const {
        size_t line = 1;
        for (size_t k = 0; k < i_ && k < s_.size(); k++)
            if (s_[k] == '\n') line++;
        raise(what + " (line " + std::to_string(line) + ")");
    }

    JValue value() {
        skip_ws();
        if (i_ >= s_.size()) fail("unexpected end of text");
        char c = s_[i_];
        if (c == '{' || c == '[') {
            if (++depth_ > 512) fail("containers nested too deeply");
            JValue v = (c == '{') ? dict() : array();
            depth_--;
            return v;
        }
        if (c == '"') {
            JValue v;
            v.kind = JValue::STR;
            v.str = string();
            return v;
        }
        if (c == '}' || c == ']' || c == ',' || c == ':') fail(std::string("unexpected '") + c + "'");
        return token();
    }

    std::string string() {
        i_++;  // opening quote
        std::string out;
        while (true) {
            if (i_ >= s_.size()) fail("unterminated string");
            char c = s_[i_++];
            if (c == '"') break;
            if (c == '\\' && i_ < s_.size()) {
                char e = s_[i_];
                const char *from = "\"\\/bfnrt";
                const char *to = "\"\\/\b\f\n\r\t";
                const char *hit = std::strchr(from, e);
                if (e != 0 && hit != nullptr) {
                    out.push_back(to[hit - from]);
                    i_++;
                    continue;
                }
            }
            out.push_back(c);
        }
        return out;
    }

    // A bare token: true / false / null, or a number read as the longest decimal prefix.
    JValue token() {
        size_t b = i_;
        while (i_ < s_.size() && !ws(s_[i_]) && !structural(s_[i_])) i_++;
        std::string t = s_.substr(b, i_ - b);
        JValue v;
        if (t == "true" || t == "false") {
            v.kind = JValue::BOOL;
            v.b = (t == "true");
            return v;
        }
        if (t == "null") return v;
        size_t k = 0;
        if (k < t.size() && (t[k] == '+' || t[k] == '-')) k++;
        size_t digits = 0;
        while (k < t.size() && t[k] >= '0' && t[k] <= '9') k++, digits++;
        if (k < t.size() && t[k] == '.') {
            k++;
            while (k < t.size() && t[k] >= '0' && t[k] <= '9') k++, digits++;
        }
        if (digits == 0) fail("could not categorise token '" + t + "'");
        if (k < t.size() && (t[k] == 'e' || t[k] == 'E')) {
            size_t e = k + 1;
            if (e < t.size() && (t[e] == '+' || t[e] == '-')) e++;
            size_t ed = 0;
            while (e < t.size() && t[e] >= '0' && t[e] <= '9') e++, ed++;
            if (ed > 0) k = e;
        }
        v.kind = JValue::NUM;
        v.num = std::strtod(t.substr(0, k).c_str(), nullptr);
        return v;
    }

    JValue array() {
        i_++;
        JValue v;
        v.kind = JValue::ARR;
        skip_ws();
        if (i_ < s_.size() && s_[i_] == ']') {
            i_++;
            return v;
        }
        while (true) {
            v.arr.push_back(value());
            skip_ws();
            if (i_ >= s_.size()) fail("unterminated array");
            if (s_[i_] == ',') {
                i_++;
                continue;
            }
            if (s_[i_] == ']') {
                i_++;
                return v;
            }
            fail("array elements must be separated by ','");
        }
    }

    JValue dict() {
        i_++;
        JValue v;
        v.kind = JValue::DICT;
        skip_ws();
        if (i_ < s_.size() && s_[i_] == '}') {
            i_++;
            return v;
        }
        while (true) {
            skip_ws();
            if (i_ >= s_.size() || s_[i_] != '"') fail("dictionary keys must be strings");
            std::string key = string();
            skip_ws();
            if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':' after a key");
            i_++;
            JValue item = value();
            if (v.has(key.c_str())) fail("dictionary has a duplicate entry for '" + key + "'");
            v.dict.emplace_back(std::move(key), std::move(item));
            skip_ws();
            if (i_ >= s_.size()) fail("unterminated dictionary");
            if (s_[i_] == ',') {
                i_++;
                continue;
            }
            if (s_[i_] == '}') {
                i_++;
                return v;
            }
            fail("expected ',' after a key : value pair");
        }
    }
};

// ---- value helpers ------------------------------------------------------------------------------
const JValue &as_dict(const JValue &v, const std::string &what) {
    if (v.kind != JValue::DICT) raise(what + " has to be a dictionary");
    return v;
}
const JValue &as_array(const JValue &v, const std::string &what) {
    if (v.kind != JValue::ARR) raise(what + " has to be an array");
    return v;
}
const std::string &as_string(const JValue &v, const std::string &what) {
    if (v.kind != JValue::STR) raise(what + " has to be a string");
    return v.str;
}
float as_float(const JValue &v, const std::string &what) {
    if (v.kind != JValue::NUM) raise(what + " has to be a number");
    return (float)v.num;
}
int as_int(const JValue &v, const std::string &what) {
    if (v.kind != JValue::NUM) raise(what + " has to be a number");
    if (!(v.num > (double)INT_MIN - 1.0 && v.num < (double)INT_MAX + 1.0)) raise(what + " is out of range");
    return (int)v.num;
}
bool as_bool(const JValue &v, const std::string &what) {
    if (v.kind != JValue::BOOL) raise(what + " has to be a boolean");
    return v.b;
}

// ---- vectors and transforms -----------------------------------------------------------------------
struct V {
    float x, y, z;
};
V vadd(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
V vsub(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
V vmulf(V a, float f) { return V{a.x * f, a.y * f, a.z * f}; }
V vhad(V a, V b) { return V{a.x * b.x, a.y * b.y, a.z * b.z}; }
V vdivv(V a, V b) { return V{a.x / b.x, a.y / b.y, a.z / b.z}; }
float vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V vnormalized(V a) {
    float im = 1 / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return V{a.x * im, a.y * im, a.z * im};
}

// Vector3::fromDson: an array whose first three NUMBER entries are x, y, z (others skipped, missing 0).
V vector_from(const JValue &v, const std::string &what) {
    if (v.kind != JValue::ARR) raise(what + ": a vector can only be read from an array");
    float c[3] = {0.0f, 0.0f, 0.0f};
    int n = 0;
    for (const JValue &e : v.arr)
        if (e.kind == JValue::NUM) {
            if (n < 3) c[n] = (float)e.num;
            n++;
        }
    return V{c[0], c[1], c[2]};
}

const float kRadian = 57.29577951308233f;

// Rotates v1 and v2 about `axis` by `angle` radians (all three unit and orthogonal).
void rotate_two(V axis, V &v1, V &v2, float angle) {
    float s = std::sin(angle), c = std::cos(angle);
    float cx = axis.y * v1.z - v1.y * axis.z, cy = v1.x * axis.z - axis.x * v1.z, cz = axis.x * v1.y - v1.x * axis.y;
    v1 = V{v1.x * c - cx * s, v1.y * c - cy * s, v1.z * c - cz * s};
    cx = axis.y * v2.z - v2.y * axis.z;
    cy = v2.x * axis.z - axis.x * v2.z;
    cz = axis.x * v2.y - v2.x * axis.y;
    v2 = V{v2.x * c - cx * s, v2.y * c - cy * s, v2.z * c - cz * s};
}

struct Xf {
    V pos{0, 0, 0}, euler{0, 0, 0}, scale{1, 1, 1};
    V tx{1, 0, 0}, ty{0, 1, 0}, tz{0, 0, 1};  // rows of the point transform (scale folded in)

    Xf() { rebake(); }
    void rebake() {
        tx = V{1, 0, 0};
        ty = V{0, 1, 0};
        tz = V{0, 0, 1};
        float fi = 1 / kRadian;
        V r = vmulf(euler, fi);
        rotate_two(ty, tx, tz, -r.y);
        rotate_two(tx, ty, tz, -r.x);
        rotate_two(tz, tx, ty, -r.z);
        tx = vhad(tx, scale);
        ty = vhad(ty, scale);
        tz = vhad(tz, scale);
    }
    V right() const { return vdivv(tx, scale); }
    V up() const { return vdivv(ty, scale); }
    V front() const { return vdivv(tz, scale); }
    V point(V v) const { return V{vdot(v, tx) + pos.x, vdot(v, ty) + pos.y, vdot(v, tz) + pos.z}; }
};

Xf transform_from(const JValue &v) {
    if (v.kind != JValue::DICT) raise("a transform can only be read from a dictionary");
    Xf t;
    if (const JValue *p = v.get("position")) t.pos = vector_from(*p, "transform position");
    if (const JValue *p = v.get("rotation")) {
        t.euler = vector_from(*p, "transform rotation");
        t.rebake();
    }
    if (const JValue *p = v.get("scale")) {
        t.scale = vector_from(*p, "transform scale");
        t.rebake();
    }
    if (const JValue *p = v.get("relative_position")) {
        V r = vector_from(*p, "transform relative_position");
        V delta = vadd(vadd(vmulf(t.right(), r.x), vmulf(t.up(), r.y)), vmulf(t.front(), r.z));
        t.pos = vadd(t.pos, delta);
    }
    return t;
}

// ---- the scene being built ----------------------------------------------------------------------
struct Face {
    float v[9];
    float n[9];
    float uv[6];  // corner texture coordinates (BakedTriFace::tex x / y)
};
struct Tex {
    int w = 0, h = 0, filter = DR_FILTER_BILINEAR;
    std::vector<float> rgba;
};
struct Unit {
    Face f;
    int mat;
};

// BakedTriFace >> Transform: vertices through the point transform, normals too with the position
// taken off again.
void transform_face(Face &f, const Xf &t) {
    for (int k = 0; k < 3; k++) {
        V p = t.point(V{f.v[3 * k], f.v[3 * k + 1], f.v[3 * k + 2]});
        V q = vsub(t.point(V{f.n[3 * k], f.n[3 * k + 1], f.n[3 * k + 2]}), t.pos);
        f.v[3 * k] = p.x, f.v[3 * k + 1] = p.y, f.v[3 * k + 2] = p.z;
        f.n[3 * k] = q.x, f.n[3 * k + 1] = q.y, f.n[3 * k + 2] = q.z;
    }
}

struct ObjFile {
    std::vector<std::string> order;  // distinct object names in file order
    std::map<std::string, std::vector<Face>> objects;  // a repeated name keeps its last object
};

struct Item {
    std::string file, object;
    Xf transform;
    int mat = -1;
};
struct SubGroup {
    std::string group;
    Xf transform;
    int fallback = -1, override_ = -1;
};
struct Group {
    std::vector<Item> items;
    std::vector<SubGroup> subgroups;
    Xf transform;
    int fallback = -1, override_ = -1;
};

bool file_opens(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

std::string read_file(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) raise("could not open file \"" + path + "\"");
    std::string text;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    std::fclose(f);
    return text;
}

class Loader {
  public:
    std::vector<dr_material> materials;
    std::vector<dr_light> lights;
    std::vector<Unit> units;
    std::vector<Tex> textures;
    int lens = -1;  // -1: none set yet
    float lens_angle[2] = {60.0f, 60.0f}, lens_focal = 128.0f, lens_soft = 1.0f, lens_filter[3] = {1, 1, 1};
    Xf camera;
    int boxing = DR_BOXING_HEIGHT, bounces = 2, spp_x = 1, spp_y = 1, pixels_per_thread = 1;
    bool ignore_backfaces = true;

    void from_file(const std::string &path, int depth = 0) {
        if (depth > 64) raise("includes nested too deeply at \"" + path + "\"");
        std::string text = read_file(path);
        JValue doc;
        try {
            doc = JParser(text).parse_document();
        } catch (const LoadError &e) {
            raise("could not parse \"" + path + "\": " + e.msg);
        }
        std::string saved = source_;
        size_t len = path.size();
        while (len > 0 && path[len - 1] != '/' && path[len - 1] != '\\') len--;
        source_ = path.substr(0, len);
        from_doc(doc, depth);
        source_ = saved;
    }

  private:
    std::string source_;  // directory of the file being read (with its trailing separator)
    std::unordered_map<std::string, int> material_names_;
    std::unordered_map<std::string, int> texture_names_;  // "name::" / "png::" keys, as the reference keeps them
    std::map<std::string, ObjFile> obj_files_;
    std::map<std::string, Group> groups_;

    std::string resolve(const std::string &name) const {
        std::string rel = source_ + name;
        return file_opens(rel) ? rel : name;
    }

    void from_doc(const JValue &doc, int depth) {
        if (doc.kind != JValue::DICT) raise("a scene can only be built from a dictionary");
        if (const JValue *v = doc.get("include")) {
            for (const JValue &e : as_array(*v, "include").arr)
                from_file(resolve(as_string(e, "an include entry")), depth + 1);
        }
        if (const JValue *v = doc.get("materials"))
            for (const JValue &e : as_array(*v, "materials").arr) parse_material(e);
        if (const JValue *v = doc.get("lights"))
            for (const JValue &e : as_array(*v, "lights").arr) parse_light(e);
        if (const JValue *v = doc.get("groups"))
            for (const JValue &e : as_array(*v, "groups").arr) parse_group(e);
        if (const JValue *v = doc.get("objects"))
            for (const JValue &e : as_array(*v, "objects").arr) parse_object(e);
        if (const JValue *v = doc.get("camera")) parse_camera(*v);
        if (lens < 0) {
            lens = DR_LENS_SIMPLE_STOCHASTIC;
            lens_angle[0] = 64.0f;
        }
        if (const JValue *v = doc.get("renderer")) parse_renderer(*v);
    }

    // ---- materials ----
    int parse_material(const JValue &v) {
        as_dict(v, "a material");
        const JValue *type = v.get("type");
        if (!type) raise("a material has to have a type");
        const std::string &t = as_string(*type, "material type");
        dr_material m;
        std::memset(&m, 0, sizeof(m));
        if (t == "dumb_based") dumb_based(v, m);
        else if (t == "simple_stochastic") simple_stochastic(v, m);
        else if (t == "fresnel_color") fresnel_color(v, m);
        else raise("unknown material type: \"" + t + "\"");
        int id = (int)materials.size();
        materials.push_back(m);
        if (const JValue *n = v.get("name"))
            if (n->kind == JValue::STR) material_names_[n->str] = id;
        return id;
    }

    // DumbRenderContext::getImageId (DumbRenderContext.cu:374-450): -1 for null / bool / number; a
    // string names a texture ("name::" then "png::" keys); a dictionary loads its "png" file (path
    // relative to the scene file first), with "filtering" and "name".  Returns the 0-based id.
    int image_id(const JValue &v) {
        if (v.kind == JValue::BOOL || v.kind == JValue::NUL || v.kind == JValue::NUM) return -1;
        if (v.kind == JValue::STR) {
            auto it = texture_names_.find("name::" + v.str);
            if (it == texture_names_.end()) it = texture_names_.find("png::" + v.str);
            if (it == texture_names_.end()) raise("texture \"" + v.str + "\" not found");
            return it->second;
        }
        if (v.kind != JValue::DICT) raise("unsupported value for a texture");
        const JValue *png = v.get("png");
        if (!png) raise("image dict incomplete");
        const std::string &file = as_string(*png, "image 'png' entry");
        const std::string path = resolve(file);
        int32_t w = 0, h = 0;
        if (dr_png_read(path.c_str(), &w, &h, nullptr) != DR_OK) raise("could not read file: \"" + path + "\"");
        std::vector<uint8_t> px((size_t)w * h * 4);
        if (dr_png_read(path.c_str(), &w, &h, px.data()) != DR_OK) raise("could not read file: \"" + path + "\"");
        Tex t;
        t.w = w;
        t.h = h;
        t.rgba.resize(px.size());
        for (size_t k = 0; k < px.size(); k++) t.rgba[k] = (((float)px[k]) / 255.0f);
        const int id = (int)textures.size();
        textures.push_back(std::move(t));
        texture_names_["png::" + path] = id;
        texture_names_["png::" + file] = id;
        if (const JValue *f = v.get("filtering")) {
            const std::string &filter = as_string(*f, "image 'filtering' entry");
            if (filter == "none") textures[(size_t)id].filter = DR_FILTER_NONE;
            else if (filter == "bilinear") textures[(size_t)id].filter = DR_FILTER_BILINEAR;
            else raise("image filter can be only \"none\"/[\"bilinear\"] (got: \"" + filter + "\")");
        }
        if (const JValue *n = v.get("name")) texture_names_["name::" + as_string(*n, "image name entry")] = id;
        return id;
    }

    // ColoredTexture::fromDson (DumbStructs.cu:7-37): colour, texture, tiling, offset entries of one
    // channel of `m` (texture ids stored 1-based, tiling and offset as the first two numbers).
    void colored(const JValue &v, const char *color_key, const char *texture_key, const char *tiling_key,
                 const char *offset_key, V &color, dr_material &m, int ch) {
        if (const JValue *c = v.get(color_key)) color = vector_from(*c, color_key);
        if (const JValue *t = v.get(texture_key)) m.texture[ch] = image_id(*t) + 1;
        if (const JValue *t = v.get(tiling_key)) {
            V x = vector_from(*t, tiling_key);
            m.tiling[ch][0] = x.x, m.tiling[ch][1] = x.y;
        }
        if (const JValue *t = v.get(offset_key)) {
            V x = vector_from(*t, offset_key);
            m.offset[ch][0] = x.x, m.offset[ch][1] = x.y;
        }
    }
    static void untextured(dr_material &m) {
        for (int k = 0; k < 4; k++) {
            m.texture[k] = 0;
            m.tiling[k][0] = m.tiling[k][1] = 1.0f;
            m.offset[k][0] = m.offset[k][1] = 0.0f;
        }
        m.normal_color[0] = m.normal_color[1] = m.normal_color[2] = 1.0f;
        m.alpha_threshold = 0.5f;
    }

    // DumbBasedShader constructor state: fresnel, spec, diffuse (scaled by 1 - metal), metal.
    struct DumbState {
        V fresnel, diffuse;
        float spec, metal;
    };
    static DumbState dumb_ctor(V fresnel, float spec, V diffuse, float metal) {
        metal = std::fmax(std::fmin(metal, 1.0f), 0.0f);
        return DumbState{fresnel, vmulf(diffuse, 1.0f - metal), spec, metal};
    }

    void dumb_based(const JValue &v, dr_material &m) {
        DumbState s = dumb_ctor(V{0.2f, 0.2f, 0.2f}, 8.0f, V{0.2f, 0.2f, 0.2f}, 0.5f);
        if (const JValue *p = v.get("preset")) {
            const std::string &preset = as_string(*p, "dumb_based preset");
            if (preset == "rough_gold") s = dumb_ctor(V{1.022f, 0.782f, 0.344f}, 16.0f, V{1.0f, 1.0f, 1.0f}, 1.0f);
            else if (preset == "glossy_gold" || preset == "gold")
                s = dumb_ctor(V{1.022f, 0.782f, 0.344f}, 128.0f, V{1.0f, 1.0f, 1.0f}, 1.0f);
            else if (preset == "glossy_finish" || preset == "glossy")
                s = dumb_ctor(V{0.175f, 0.15f, 0.125f}, 4096.0f, V{0.32f, 0.32f, 0.32f}, 0.25f);
            else if (preset == "matte_finish" || preset == "matte")
                s = dumb_ctor(V{0.175f, 0.15f, 0.125f}, 8.0f, V{0.24f, 0.24f, 0.24f}, 0.05f);
            else raise("dumb_based preset \"" + preset + "\" does not exist");
        }
        V fresnel = s.fresnel;
        float metal = s.metal, specular = s.spec;
        float inv = 1.0f / ((metal == 1.0f) ? 1.0f : (1.0f - metal));
        V diffuse = vmulf(s.diffuse, inv);
        V normal{1.0f, 1.0f, 1.0f}, cutout{1.0f, 1.0f, 1.0f};
        untextured(m);
        colored(v, "fresnel", "fresnel_texture", "fresnel_tiling", "fresnel_offset", fresnel, m, DR_TEX_FRESNEL);
        colored(v, "diffuse", "diffuse_texture", "diffuse_tiling", "diffuse_offset", diffuse, m, DR_TEX_COLOR);
        colored(v, "normal_color", "normal_texture", "normal_tiling", "normal_offset", normal, m, DR_TEX_NORMAL);
        colored(v, "alpha_cutout_color", "alpha_cutout_texture", "alpha_cutout_tiling", "alpha_cutout_offset", cutout, m,
                DR_TEX_ALPHA);
        if (const JValue *p = v.get("alpha_cutout_threshold")) m.alpha_threshold = as_float(*p, "dumb_based alpha_cutout_threshold");
        if (const JValue *p = v.get("specular")) specular = as_float(*p, "dumb_based specular");
        if (const JValue *p = v.get("metal")) metal = as_float(*p, "dumb_based metal");
        m.normal_color[0] = normal.x, m.normal_color[1] = normal.y, m.normal_color[2] = normal.z;
        m.type = DR_MAT_DUMB_BASED;
        m.fresnel[0] = fresnel.x, m.fresnel[1] = fresnel.y, m.fresnel[2] = fresnel.z;
        m.color[0] = diffuse.x, m.color[1] = diffuse.y, m.color[2] = diffuse.z;
        m.specular = specular;
        m.metal = metal;
    }

    void simple_stochastic(const JValue &v, dr_material &m) {
        untextured(m);
        // constructor state of SimpleStochasticShader() = ((1,1,1), 0.05, 0.95, 2)
        float total = 0.05f + 0.95f;
        float mul = ((total > 1.0f) ? (1.0f / total) : 1.0f);
        V color{1.0f, 1.0f, 1.0f};
        float diffuse = 0.05f * mul, smoothness = 0.95f * mul, shininess = 2.0f;
        if (const JValue *p = v.get("color")) color = vector_from(*p, "simple_stochastic color");
        if (const JValue *p = v.get("diffuse")) diffuse = as_float(*p, "simple_stochastic diffuse");
        if (const JValue *p = v.get("smoothness")) smoothness = as_float(*p, "simple_stochastic smoothness");
        if (const JValue *p = v.get("shininess")) shininess = as_float(*p, "simple_stochastic shininess");
        m.type = DR_MAT_SIMPLE_STOCHASTIC;
        m.color[0] = color.x, m.color[1] = color.y, m.color[2] = color.z;
        m.diffuse = diffuse;
        m.smoothness = smoothness;
        m.shininess = shininess;
    }

    // Shaders::FresnelShader::fromDson (FresnelShader.impl.cuh:20-24): white, then an "engine_color"
    // preset (DumbStructs.cuh:143-169; the reference ignores a bad one), then the colour entries.
    void fresnel_color(const JValue &v, dr_material &m) {
        untextured(m);
        V color{1.0f, 1.0f, 1.0f};
        if (const JValue *e = v.get("engine_color")) {
            if (e->kind == JValue::STR) {
                const std::string &n = e->str;
                if (n == "iron") color = V{0.56f, 0.57f, 0.58f};
                else if (n == "copper") color = V{0.95f, 0.64f, 0.54f};
                else if (n == "gold") color = V{1.0f, 0.71f, 0.29f};
                else if (n == "aluminum") color = V{0.91f, 0.92f, 0.92f};
                else if (n == "silver") color = V{0.95f, 0.93f, 0.88f};
            }
        }
        colored(v, "color", "texture", "tiling", "offset", color, m, DR_TEX_COLOR);
        m.type = DR_MAT_FRESNEL;
        m.color[0] = color.x, m.color[1] = color.y, m.color[2] = color.z;
    }

    int material_ref(const JValue &v) {
        if (v.kind == JValue::STR) {
            auto it = material_names_.find(v.str);
            if (it == material_names_.end()) raise("material not found: \"" + v.str + "\"");
            return it->second;
        }
        return parse_material(v);
    }

    // ---- lights ----
    void parse_light(const JValue &v) {
        as_dict(v, "a light");
        const JValue *type = v.get("type");
        if (!type) raise("a light has to have a type");
        const std::string &t = as_string(*type, "light type");
        dr_light l;
        std::memset(&l, 0, sizeof(l));
        if (t == "simple_soft_directional") {
            // constructor state of SimpleSoftDirectionalLight(): colour 1, direction (1,-1,1) normalised
            // (and normalised again by the constructor), distance 1024, soft = 1024 * 0.125
            V color{1.0f, 1.0f, 1.0f};
            V dir = vnormalized(vnormalized(V{1.0f, -1.0f, 1.0f}));
            float dist = 1024.0f, soft = dist * 0.125f;
            float distance = dist;
            float softness = (soft / ((distance == 0.0f) ? 0.0f : distance));
            if (const JValue *p = v.get("color")) color = vector_from(*p, "simple_soft_directional color");
            if (const JValue *p = v.get("direction")) dir = vector_from(*p, "simple_soft_directional direction");
            if (const JValue *p = v.get("distance")) distance = as_float(*p, "simple_soft_directional distance");
            if (const JValue *p = v.get("softness")) softness = as_float(*p, "simple_soft_directional softness");
            l.type = DR_LIGHT_SOFT_DIRECTIONAL;
            l.color[0] = color.x, l.color[1] = color.y, l.color[2] = color.z;
            l.direction[0] = dir.x, l.direction[1] = dir.y, l.direction[2] = dir.z;
            l.distance = distance;
            l.softness = softness;
        } else if (t == "simple_spherical") {
            V color{1.0f, 1.0f, 1.0f}, position{0.0f, 0.0f, 0.0f};
            float radius = 1.0f;
            if (const JValue *p = v.get("color")) color = vector_from(*p, "simple_spherical color");
            if (const JValue *p = v.get("position")) position = vector_from(*p, "simple_spherical position");
            if (const JValue *p = v.get("radius")) radius = as_float(*p, "simple_spherical radius");
            l.type = DR_LIGHT_SPHERICAL;
            l.color[0] = color.x, l.color[1] = color.y, l.color[2] = color.z;
            l.position[0] = position.x, l.position[1] = position.y, l.position[2] = position.z;
            l.radius = radius;
        } else if (t == "spotlight") {
            spotlight(v, l);
        } else {
            raise("unknown light type: \"" + t + "\"");
        }
        lights.push_back(l);
    }

    // Lights::Spotlight::fromDson (Spotlight.impl.cuh:79-151): constructor arguments with their
    // defaults; "target" (minus the position read so far) wins over "direction"; an unknown
    // "emitter_shape" keeps the disc (the reference only reports it).
    static void spotlight(const JValue &v, dr_light &l) {
        V color{1.0f, 1.0f, 1.0f}, pos{0.0f, 0.0f, 0.0f}, dir{0.0f, 0.0f, 1.0f};
        float lum = 1500.0f, inner = 16.0f, outer = 64.0f, power = 1.0f, size = 0.25f;
        bool sphere = false, shadows = true;
        int samples = 1;
        if (const JValue *p = v.get("color")) color = vector_from(*p, "spotlight color");
        if (const JValue *p = v.get("luminosity")) lum = as_float(*p, "spotlight luminosity");
        if (const JValue *p = v.get("position")) pos = vector_from(*p, "spotlight position");
        if (const JValue *p = v.get("target")) dir = vsub(vector_from(*p, "spotlight target"), pos);
        else if (const JValue *p = v.get("direction")) dir = vector_from(*p, "spotlight direction");
        if (const JValue *p = v.get("hotspot_angle")) inner = as_float(*p, "spotlight hotspot angle");
        if (const JValue *p = v.get("falloff_angle")) outer = as_float(*p, "spotlight falloff angle");
        if (const JValue *p = v.get("falloff_power")) power = as_float(*p, "spotlight falloff power");
        if (const JValue *p = v.get("emitter_size")) size = as_float(*p, "spotlight emitter size");
        if (const JValue *p = v.get("emitter_shape")) {
            const std::string &shape = as_string(*p, "spotlight emitter shape");
            if (shape == "sphere") sphere = true;
            else if (shape == "disc") sphere = false;
        }
        if (const JValue *p = v.get("cast_shadows")) shadows = as_bool(*p, "spotlight shadow cast flag");
        if (const JValue *p = v.get("sample_count")) samples = as_int(*p, "spotlight sample count");
        l.type = DR_LIGHT_SPOTLIGHT;
        l.color[0] = color.x, l.color[1] = color.y, l.color[2] = color.z;
        l.position[0] = pos.x, l.position[1] = pos.y, l.position[2] = pos.z;
        l.direction[0] = dir.x, l.direction[1] = dir.y, l.direction[2] = dir.z;
        l.luminosity = lum;
        l.hotspot_angle = inner;
        l.falloff_angle = outer;
        l.falloff_power = power;
        l.emitter_size = size;
        l.emit_from_sphere = sphere ? 1 : 0;
        l.cast_shadows = shadows ? 1 : 0;
        l.samples = samples;
    }

    // ---- meshes, items, groups, objects ----
    const ObjFile &load_obj(const std::string &name) {
        auto it = obj_files_.find(name);
        if (it != obj_files_.end()) return it->second;
        std::string path = resolve(name);
        dr_mesh_file *mf = nullptr;
        if (dr_obj_read(path.c_str(), &mf) != DR_OK)
            raise("could not read file: '" + name + "' (" + path + "): " + dr_last_error());
        ObjFile of;
        for (int32_t i = 0; i < dr_mesh_file_objects(mf); i++) {
            std::string oname = dr_mesh_file_object_name(mf, i);
            int32_t n = dr_mesh_file_object_triangles(mf, i);
            std::vector<float> xyz((size_t)n * 9), nrm((size_t)n * 9), uvw((size_t)n * 9);
            dr_mesh_file_object_data(mf, i, xyz.data(), nrm.data(), uvw.data());
            std::vector<Face> faces((size_t)n);
            for (int32_t k = 0; k < n; k++) {
                std::memcpy(faces[k].v, &xyz[(size_t)k * 9], sizeof(float) * 9);
                std::memcpy(faces[k].n, &nrm[(size_t)k * 9], sizeof(float) * 9);
                for (int c = 0; c < 3; c++) {
                    faces[k].uv[2 * c] = uvw[(size_t)k * 9 + 3 * c];
                    faces[k].uv[2 * c + 1] = uvw[(size_t)k * 9 + 3 * c + 1];
                }
            }
            if (of.objects.find(oname) == of.objects.end()) of.order.push_back(oname);
            of.objects[oname] = std::move(faces);
        }
        dr_mesh_file_destroy(mf);
        return obj_files_.emplace(name, std::move(of)).first->second;
    }

    Item parse_item(const JValue &v) {
        as_dict(v, "a group item");
        Item item;
        const JValue *mesh = v.get("mesh");
        if (!mesh) raise("an item has to have a 'mesh' entry");
        as_dict(*mesh, "an item 'mesh' entry");
        if (const JValue *f = mesh->get("obj")) {
            item.file = as_string(*f, ".obj file name");
            load_obj(item.file);
        } else if (mesh->has("primitive")) {
            raise("mesh primitives are not supported (the reference leaves them unimplemented)");
        } else {
            raise("object mesh could not be parsed");
        }
        if (const JValue *o = mesh->get("object")) {
            item.object = as_string(*o, ".obj mesh name");
            const ObjFile &of = obj_files_.at(item.file);
            if (of.objects.find(item.object) == of.objects.end())
                raise("object [" + item.object + "] not found in [" + item.file + "]");
        }
        if (const JValue *t = v.get("transform")) item.transform = transform_from(*t);
        if (const JValue *m = v.get("material")) item.mat = material_ref(*m);
        return item;
    }

    std::vector<Unit> resolve_item(const Item &item) const {
        std::vector<Unit> out;
        const ObjFile &of = obj_files_.at(item.file);
        auto emit = [&](const std::vector<Face> &faces) {
            for (const Face &f : faces) {
                Unit u{f, item.mat};
                transform_face(u.f, item.transform);
                out.push_back(u);
            }
        };
        if (!item.object.empty()) emit(of.objects.at(item.object));
        else
            for (const std::string &n : of.order) emit(of.objects.at(n));
        return out;
    }

    SubGroup parse_subgroup(const JValue &v) {
        SubGroup sg;
        if (v.kind == JValue::STR) {
            sg.group = "named::" + v.str;
            if (groups_.find(sg.group) == groups_.end()) raise("group [" + v.str + "] not found");
            return sg;
        }
        as_dict(v, "a subgroup (a string or a dictionary)");
        if (const JValue *g = v.get("group")) {
            sg.group = "named::" + as_string(*g, "a subgroup's 'group' entry");
            if (groups_.find(sg.group) == groups_.end()) raise("group [" + sg.group + "] not found");
            if (const JValue *t = v.get("transform")) sg.transform = transform_from(*t);
            if (const JValue *m = v.get("fallback_material")) sg.fallback = material_ref(*m);
            if (const JValue *m = v.get("override_material")) sg.override_ = material_ref(*m);
        } else {
            sg.group = parse_group(v);
        }
        return sg;
    }

    std::string parse_group(const JValue &v) {
        as_dict(v, "a group");
        Group g;
        if (const JValue *e = v.get("elements")) {
            for (const JValue &el : as_array(*e, "group elements").arr) {
                if (el.kind == JValue::DICT && el.has("mesh")) g.items.push_back(parse_item(el));
                else g.subgroups.push_back(parse_subgroup(el));
            }
        }
        if (const JValue *t = v.get("transform")) g.transform = transform_from(*t);
        if (const JValue *m = v.get("fallback_material")) g.fallback = material_ref(*m);
        if (const JValue *m = v.get("override_material")) g.override_ = material_ref(*m);
        std::string name;
        if (const JValue *n = v.get("name")) name = "named::" + as_string(*n, "group name");
        else name = "unnamed::" + std::to_string(groups_.size());
        groups_[name] = g;
        return name;
    }

    static void finish(std::vector<Unit> &units, int override_, int fallback, const Xf &t) {
        for (Unit &u : units) {
            if (override_ >= 0) u.mat = override_;
            else if (u.mat < 0) u.mat = fallback;
            transform_face(u.f, t);
        }
    }

    std::vector<Unit> resolve_group(const std::string &name, int depth) const {
        if (depth > 256) raise("groups nested too deeply");
        const Group &g = groups_.at(name);
        std::vector<Unit> out;
        for (const Item &it : g.items) {
            std::vector<Unit> add = resolve_item(it);
            out.insert(out.end(), add.begin(), add.end());
        }
        for (const SubGroup &sg : g.subgroups) {
            std::vector<Unit> add = resolve_subgroup(sg, depth + 1);
            out.insert(out.end(), add.begin(), add.end());
        }
        finish(out, g.override_, g.fallback, g.transform);
        return out;
    }

    std::vector<Unit> resolve_subgroup(const SubGroup &sg, int depth) const {
        std::vector<Unit> out = resolve_group(sg.group, depth);
        finish(out, sg.override_, sg.fallback, sg.transform);
        return out;
    }

    void parse_object(const JValue &v) {
        if (v.kind == JValue::DICT && v.has("mesh")) {
            Item item = parse_item(v);
            if (item.mat < 0) raise("an object must have a material attached to it");
            std::vector<Unit> add = resolve_item(item);
            units.insert(units.end(), add.begin(), add.end());
        } else {
            SubGroup sg = parse_subgroup(v);
            std::vector<Unit> add = resolve_subgroup(sg, 0);
            for (const Unit &u : add)
                if (u.mat < 0) raise("a resolved group must have a material attached to it");
            units.insert(units.end(), add.begin(), add.end());
        }
    }

    // ---- camera and renderer ----
    void parse_camera(const JValue &v) {
        as_dict(v, "the camera");
        if (const JValue *l = v.get("lense")) {
            if (l->kind != JValue::DICT) raise("the camera lense has to be a dictionary");
            const JValue *type = l->get("type");
            if (!type) raise("a lense has to have a type");
            const std::string &t = as_string(*type, "lense type");
            if (t == "simple_stochastic") {
                float angle = 60.0f;
                if (const JValue *a = l->get("angle")) angle = as_float(*a, "simple_stochastic lense angle");
                lens = DR_LENS_SIMPLE_STOCHASTIC;
                lens_angle[0] = angle;
                lens_angle[1] = angle;
            } else if (t == "spherical_segment") {
                float a0 = 60.0f, a1 = 60.0f, dist = 128.0f, soft = 1.0f;
                V filter{1.0f, 1.0f, 1.0f};
                if (const JValue *a = l->get("angle")) a0 = a1 = as_float(*a, "spherical_segment angle");
                if (const JValue *a = l->get("distance")) dist = as_float(*a, "spherical_segment distance");
                if (const JValue *a = l->get("sensor")) soft = as_float(*a, "spherical_segment sensor size");
                if (const JValue *a = l->get("filter")) filter = vector_from(*a, "spherical_segment filter");
                lens = DR_LENS_SPHERICAL_SEGMENT;
                lens_angle[0] = a0;
                lens_angle[1] = a1;
                lens_focal = dist;
                lens_soft = soft;
                lens_filter[0] = filter.x, lens_filter[1] = filter.y, lens_filter[2] = filter.z;
            } else {
                raise("unknown lense type: \"" + t + "\"");
            }
        }
        if (const JValue *t = v.get("transform")) camera = transform_from(*t);
    }

    void parse_renderer(const JValue &v) {
        as_dict(v, "the renderer");
        if (const JValue *r = v.get("resources")) {
            as_dict(*r, "renderer resources");
            if (const JValue *c = r->get("cpu")) {
                if (c->kind == JValue::STR) {
                    const std::string &s = c->str;
                    if (s != "all" && s != "all_but_gpu" && s != "all_but_one_per_gpu" && s != "none" && s != "one")
                        raise("renderer resources cpu can only be one of 'all'/['all_but_gpu']/'all_but_one_per_gpu'/'none'/'one'/any_number");
                } else if (c->kind != JValue::NUM) {
                    raise("renderer resources cpu can only be one of 'all'/['all_but_gpu']/'all_but_one_per_gpu'/'none'/'one'/any_number");
                }
            }
            if (const JValue *g = r->get("gpu")) as_int(*g, "renderer resources gpu");
            // one device per process: the per-device entry that exists is gpu_0
            if (const JValue *g = r->get("gpu_0")) as_int(*g, "renderer resources gpu_0");
        }
        if (const JValue *b = v.get("blocks")) {
            as_dict(*b, "renderer blocks");
            if (const JValue *x = b->get("cpu_cut")) as_int(*x, "renderer blocks cpu_cut");
            if (const JValue *x = b->get("gpu_cut")) as_int(*x, "renderer blocks gpu_cut");
            if (const JValue *x = b->get("force_host_block_synchronisation"))
                as_bool(*x, "renderer blocks force_host_block_synchronisation");
        }
        if (const JValue *p = v.get("pixel")) {
            as_dict(*p, "renderer pixel");
            if (const JValue *x = p->get("boxing")) {
                const std::string &s = as_string(*x, "renderer pixel boxing");
                if (s == "height") boxing = DR_BOXING_HEIGHT;
                else if (s == "width") boxing = DR_BOXING_WIDTH;
                else if (s == "min") boxing = DR_BOXING_MIN;
                else if (s == "max") boxing = DR_BOXING_MAX;
                else raise("renderer pixel boxing mode can only be one of ['height']/'width'/'min'/'max'");
            }
            if (const JValue *x = p->get("bounces")) bounces = as_int(*x, "renderer pixel bounces");
            if (const JValue *x = p->get("samples_per_pixel")) {
                if (x->kind != JValue::ARR || x->arr.size() != 2 || x->arr[0].kind != JValue::NUM || x->arr[1].kind != JValue::NUM)
                    raise("renderer pixel samples_per_pixel has to be an array, containing two numbers");
                spp_x = as_int(x->arr[0], "samples_per_pixel");
                spp_y = as_int(x->arr[1], "samples_per_pixel");
            }
            if (const JValue *x = p->get("pixels_per_gpu_thread"))
                pixels_per_thread = as_int(*x, "renderer pixel pixels_per_gpu_thread");
            if (const JValue *x = p->get("ignore_backfaces")) ignore_backfaces = as_bool(*x, "renderer pixel ignore_backfaces");
        }
    }
};

dr_status fail(dr_status s, const std::string &msg) {
    dr_internal_set_error(msg.c_str());
    return s;
}

}  // namespace

struct dr_scene_file {
    Loader L;
};

extern "C" {

dr_status dr_scene_file_load(const char *path, dr_scene_file **out) try {
    if (!out) return fail(DR_E_ARG, "dr_scene_file_load: out is NULL");
    *out = nullptr;
    if (!path) return fail(DR_E_ARG, "dr_scene_file_load: path is NULL");
    std::unique_ptr<dr_scene_file> f(new (std::nothrow) dr_scene_file());
    if (!f) return fail(DR_E_NOMEM, "dr_scene_file_load: out of host memory");
    try {
        f->L.from_file(path);
    } catch (const LoadError &e) {
        return fail(DR_E_ARG, std::string("dr_scene_file_load: ") + e.msg);
    } catch (const std::bad_alloc &) {
        return fail(DR_E_NOMEM, "dr_scene_file_load: out of host memory");
    }
    *out = f.release();
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_load");
}

dr_status dr_scene_file_counts(const dr_scene_file *f, int32_t *counts) try {
    if (!f || !counts) return fail(DR_E_ARG, "dr_scene_file_counts: NULL argument");
    counts[0] = (int32_t)f->L.units.size();
    counts[1] = (int32_t)f->L.materials.size();
    counts[2] = (int32_t)f->L.lights.size();
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_counts");
}

dr_status dr_scene_file_geometry(const dr_scene_file *f, float *xyz, float *nrm, int32_t *mat_id) try {
    if (!f) return fail(DR_E_ARG, "dr_scene_file_geometry: file is NULL");
    for (size_t i = 0; i < f->L.units.size(); i++) {
        const Unit &u = f->L.units[i];
        if (xyz) std::memcpy(xyz + 9 * i, u.f.v, sizeof(float) * 9);
        if (nrm) std::memcpy(nrm + 9 * i, u.f.n, sizeof(float) * 9);
        if (mat_id) mat_id[i] = u.mat;
    }
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_geometry");
}

dr_status dr_scene_file_materials(const dr_scene_file *f, dr_material *mats) try {
    if (!f || !mats) return fail(DR_E_ARG, "dr_scene_file_materials: NULL argument");
    if (!f->L.materials.empty()) std::memcpy(mats, f->L.materials.data(), sizeof(dr_material) * f->L.materials.size());
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_materials");
}

dr_status dr_scene_file_lights(const dr_scene_file *f, dr_light *lights) try {
    if (!f || !lights) return fail(DR_E_ARG, "dr_scene_file_lights: NULL argument");
    if (!f->L.lights.empty()) std::memcpy(lights, f->L.lights.data(), sizeof(dr_light) * f->L.lights.size());
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_lights");
}

dr_status dr_scene_file_camera(const dr_scene_file *f, dr_camera *c) try {
    if (!f || !c) return fail(DR_E_ARG, "dr_scene_file_camera: NULL argument");
    const Loader &L = f->L;
    std::memset(c, 0, sizeof(*c));
    c->lens = L.lens;
    c->angle[0] = L.lens_angle[0];
    c->angle[1] = L.lens_angle[1];
    c->focal_distance = L.lens_focal;
    c->softness = L.lens_soft;
    for (int k = 0; k < 3; k++) c->filter[k] = L.lens_filter[k];
    const Xf &t = L.camera;
    V r = t.right(), u = t.up(), fw = t.front();
    const float pos[3] = {t.pos.x, t.pos.y, t.pos.z};
    const float rr[3] = {r.x, r.y, r.z}, uu[3] = {u.x, u.y, u.z}, ff[3] = {fw.x, fw.y, fw.z};
    const float rx[3] = {t.tx.x, t.tx.y, t.tx.z}, ry[3] = {t.ty.x, t.ty.y, t.ty.z}, rz[3] = {t.tz.x, t.tz.y, t.tz.z};
    for (int k = 0; k < 3; k++) {
        c->position[k] = pos[k];
        c->right[k] = rr[k];
        c->up[k] = uu[k];
        c->forward[k] = ff[k];
        c->row_x[k] = rx[k];
        c->row_y[k] = ry[k];
        c->row_z[k] = rz[k];
    }
    c->origin_rows = 1;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_camera");
}

dr_status dr_scene_file_render_params(const dr_scene_file *f, dr_render_params *p) try {
    if (!f || !p) return fail(DR_E_ARG, "dr_scene_file_render_params: NULL argument");
    std::memset(p, 0, sizeof(*p));
    p->mode = DR_MODE_REFERENCE;
    p->samples_x = f->L.spp_x;
    p->samples_y = f->L.spp_y;
    p->max_bounces = f->L.bounces;
    p->cull_backfaces = f->L.ignore_backfaces ? 1 : 0;
    p->boxing = f->L.boxing;
    p->iteration = 1;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_render_params");
}

int32_t dr_scene_file_textures(const dr_scene_file *f) { return f ? (int32_t)f->L.textures.size() : 0; }

dr_status dr_scene_file_texture(const dr_scene_file *f, int32_t i, int32_t *width, int32_t *height, int32_t *filtering,
                                float *rgba) try {
    if (!f || i < 0 || i >= (int32_t)f->L.textures.size()) return fail(DR_E_ARG, "dr_scene_file_texture: bad texture");
    const Tex &t = f->L.textures[(size_t)i];
    if (width) *width = t.w;
    if (height) *height = t.h;
    if (filtering) *filtering = t.filter;
    if (rgba) std::memcpy(rgba, t.rgba.data(), sizeof(float) * t.rgba.size());
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_texture");
}

dr_status dr_scene_file_texcoords(const dr_scene_file *f, float *uv) try {
    if (!f || !uv) return fail(DR_E_ARG, "dr_scene_file_texcoords: NULL argument");
    for (size_t i = 0; i < f->L.units.size(); i++) std::memcpy(uv + 6 * i, f->L.units[i].f.uv, sizeof(float) * 6);
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_scene_file_texcoords");
}

dr_status dr_scene_file_create_scene(const dr_scene_file *f, const dr_build_params *bp, dr_scene **out) try {
    if (!f || !out) return fail(DR_E_ARG, "dr_scene_file_create_scene: NULL argument");
    const Loader &L = f->L;
    const size_t n = L.units.size();
    std::vector<float> xyz(n * 9), nrm(n * 9), uv(n * 6);
    std::vector<int32_t> mat(n);
    dr_scene_file_geometry(f, xyz.data(), nrm.data(), mat.data());
    dr_status st = dr_scene_create(xyz.data(), nrm.data(), mat.data(), (int32_t)n, L.materials.data(),
                                   (int32_t)L.materials.size(), L.lights.data(), (int32_t)L.lights.size(), bp, out);
    if (st != DR_OK || L.textures.empty()) return st;
    std::vector<dr_texture> tex;
    for (const Tex &t : L.textures) tex.push_back(dr_texture{t.w, t.h, t.filter, t.rgba.data()});
    if (n) dr_scene_file_texcoords(f, uv.data());
    st = dr_scene_set_textures(*out, tex.data(), (int32_t)tex.size(), uv.data());
    if (st != DR_OK) {
        dr_scene_destroy(*out);
        *out = nullptr;
    }
    return st;
} catch (...) {
    return dr_internal_exception("dr_scene_file_create_scene");
}

void dr_scene_file_destroy(dr_scene_file *f) { delete f; }

}  // extern "C"
