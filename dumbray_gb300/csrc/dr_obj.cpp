// dr_obj.cpp - Wavefront OBJ ingestion with the reference's reading rules, for scenes built from
// the same files the reference renders.
//
// Behaviour of MeshReader::readObj + PolyMesh::bake (Namespaces/MeshReader/MeshReader.impl.h:160-367,
// DataStructures/Objects/Meshes/PolyMesh/PolyMesh.impl.h:140-152), restated:
//  * statements are whitespace-separated tokens; '#' starts a comment to the end of the line;
//  * `v` and `vn` read up to three numbers from their line (missing ones are 0) and mirror x
//    (x -> -x, the reference's handedness); `vt` reads three numbers as they are;
//  * `f` reads `v[/t[/n]]` corner tokens to the end of the line (1-based; an empty field is -1);
//  * objects are the face ranges between `g` lines; the name is the rest of the `g` line with
//    trailing white space removed (`o` lines are ignored, like every other statement);
//  * every vertex gets a generated normal: the normalised sum, over the corners where it is used
//    in any face of the file, of cross(prev - cur, next - cur);
//  * per object, vertices, normals and texture coordinates are renumbered in order of first use;
//    normal / texture indices are renumbered by their file index, so all corners without a `vn`
//    (index -1; any negative index counts as missing) share the generated normal of the first such
//    corner of the object, and all corners without a `vt` share (0, 0, 0);
//  * polygons become triangle fans (0, i-1, i);
//  * the file fails to load when a corner references a missing vertex, normal or texture
//    coordinate, and (as the scene loader requires) when the number of names differs from the
//    number of objects.
// Float parsing is strtod rounded to float (the reference's atof cast to float); the normal
// arithmetic is float with the reference's operation order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cwctype>
#include <map>
#include <string>
#include <vector>

#include "../../include/dr_api.h"
#include "dr_guard.h"

void dr_internal_set_error(const char *msg);

struct V3 {
    float x, y, z;
};

struct dr_mesh_file {
    struct Object {
        std::string name;
        std::vector<float> xyz, nrm, uv;   // [tris][3][3]
    };
    std::vector<Object> objects;
};

namespace {

dr_status fail(dr_status s, const std::string &msg) {
    dr_internal_set_error(msg.c_str());
    return s;
}

struct Corner {
    int v, t, n;
};

class Reader {
  public:
    explicit Reader(const std::string &text) : s_(text) {}

    bool done() const { return i_ >= s_.size(); }

    // Next statement token.  Skips white space (new lines included); a '#' swallows its line.
    // Returns false for a comment or the end of the text.
    bool statement(std::string &tok) {
        skip_space(false);
        if (done()) return false;
        if (s_[i_] == '#') {
            rest_of_line();
            return false;
        }
        tok = word();
        return true;
    }

    // Next token on the current line (false at the end of the line, at '#' or at the end).
    bool on_line(std::string &tok) {
        if (!skip_space(true)) return false;
        if (done()) return false;
        if (s_[i_] == '#') {
            rest_of_line();
            return false;
        }
        tok = word();
        return true;
    }

    // The rest of a line after skipping leading white space (new lines included), right-trimmed.
    std::string rest_of_line() {
        skip_space(false);
        std::string out;
        while (!done() && s_[i_] != '\n') out.push_back(s_[i_++]);
        while (!out.empty() && std::iswspace((unsigned char)out.back())) out.pop_back();
        return out;
    }

  private:
    // Skips white space; with stop_at_newline, stops on '\n' and returns false there.
    bool skip_space(bool stop_at_newline) {
        while (!done() && std::iswspace((unsigned char)s_[i_])) {
            if (stop_at_newline && s_[i_] == '\n') return false;
            i_++;
        }
        return true;
    }
    std::string word() {
        std::string out;
        while (!done() && !std::iswspace((unsigned char)s_[i_])) out.push_back(s_[i_++]);
        return out;
    }
    const std::string &s_;
    size_t i_ = 0;
};

float parse_float(const std::string &t) { return (float)std::strtod(t.c_str(), nullptr); }

// "v/t/n" -> zero-based indices; an absent or empty field is -1 (atoi of the digits before '/').
Corner parse_corner(const std::string &t) {
    int f[3] = {-1, -1, -1};
    size_t pos = 0;
    for (int k = 0; k < 3; k++) {
        std::string digits;
        while (pos < t.size() && t[pos] != '/') digits.push_back(t[pos++]);
        f[k] = (digits.empty() ? 0 : std::atoi(digits.c_str())) - 1;
        pos++;   // past '/'
    }
    return Corner{f[0], f[1], f[2]};
}

V3 read_vec(Reader &r, float sx) {
    float c[3] = {0.0f, 0.0f, 0.0f};
    std::string tok;
    for (int k = 0; k < 3; k++) {
        if (!r.on_line(tok)) break;
        c[k] = parse_float(tok);
    }
    return V3{c[0] * sx, c[1], c[2]};
}

}  // namespace

extern "C" {

dr_status dr_obj_read(const char *path, dr_mesh_file **out) try {
    if (!out) return fail(DR_E_ARG, "dr_obj_read: out is NULL");
    *out = nullptr;
    if (!path) return fail(DR_E_ARG, "dr_obj_read: path is NULL");
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(DR_E_ARG, std::string("dr_obj_read: cannot open ") + path);
    std::string text;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    std::fclose(f);

    std::vector<V3> verts, norms, texs;
    std::vector<std::vector<Corner>> faces;
    std::vector<std::pair<size_t, size_t>> ranges;
    std::vector<std::string> names;
    size_t start = 0;
    Reader r(text);
    std::string tok;
    while (!r.done()) {
        if (!r.statement(tok)) continue;
        if (tok == "v") verts.push_back(read_vec(r, -1.0f));
        else if (tok == "vn") norms.push_back(read_vec(r, -1.0f));
        else if (tok == "vt") texs.push_back(read_vec(r, 1.0f));
        else if (tok == "f") {
            faces.emplace_back();
            std::string c;
            while (r.on_line(c)) faces.back().push_back(parse_corner(c));
        } else if (tok == "g") {
            // a group closes the faces read since the previous one; a group without faces drops
            // the names collected so far (the reference's bookkeeping, kept so the same files load)
            if (faces.size() > start) {
                ranges.push_back({start, faces.size()});
                start = faces.size();
            } else {
                names.clear();
            }
            names.push_back(r.rest_of_line());
        }
    }
    if (faces.size() > start) ranges.push_back({start, faces.size()});
    else names.clear();

    // generated vertex normals over every face of the file
    std::vector<V3> vn(verts.size(), V3{0.0f, 0.0f, 0.0f});
    if (!ranges.empty()) {
        for (const auto &face : faces) {
            const int m = (int)face.size();
            for (int j = 0; j < m; j++) {
                const int p = face[(j - 1 + m) % m].v, q = face[(j + 1) % m].v, c = face[j].v;
                if (p < 0 || p >= (int)verts.size() || q < 0 || q >= (int)verts.size() || c < 0 || c >= (int)verts.size())
                    return fail(DR_E_ARG, std::string("dr_obj_read: a face references a missing vertex in ") + path);
                const V3 a{verts[p].x - verts[c].x, verts[p].y - verts[c].y, verts[p].z - verts[c].z};
                const V3 b{verts[q].x - verts[c].x, verts[q].y - verts[c].y, verts[q].z - verts[c].z};
                V3 &acc = vn[c];
                acc.x += a.y * b.z - b.y * a.z;
                acc.y += b.x * a.z - a.x * b.z;
                acc.z += a.x * b.y - b.x * a.y;
            }
        }
        for (V3 &v : vn) {
            if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f) {
                const float inv = 1.0f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);   // float sqrt
                v.x *= inv;
                v.y *= inv;
                v.z *= inv;
            }
        }
    }
    if (names.size() != ranges.size())
        return fail(DR_E_ARG, std::string("dr_obj_read: ") + path + " does not have as many group names as objects");

    dr_mesh_file *M = new (std::nothrow) dr_mesh_file();
    if (!M) return fail(DR_E_NOMEM, "dr_obj_read: out of host memory");
    for (size_t k = 0; k < ranges.size(); k++) {
        dr_mesh_file::Object obj;
        obj.name = names[k];
        std::vector<V3> ov, on, ot;
        std::map<int, int> vi, ni, ti;
        std::vector<std::vector<Corner>> of;
        for (size_t fi = ranges[k].first; fi < ranges[k].second; fi++) {
            std::vector<Corner> face;
            for (const Corner &c : faces[fi]) {
                if (!vi.count(c.v)) {
                    vi[c.v] = (int)ov.size();
                    ov.push_back(verts[c.v]);
                }
                if (!ni.count(c.n)) {
                    if (c.n >= (int)norms.size()) {
                        delete M;
                        return fail(DR_E_ARG, std::string("dr_obj_read: a face references a missing normal in ") + path);
                    }
                    ni[c.n] = (int)on.size();
                    on.push_back(c.n >= 0 ? norms[c.n] : vn[c.v]);
                }
                if (!ti.count(c.t)) {
                    if (c.t >= (int)texs.size()) {
                        delete M;
                        return fail(DR_E_ARG, std::string("dr_obj_read: a face references a missing texture coordinate in ") + path);
                    }
                    ti[c.t] = (int)ot.size();
                    ot.push_back(c.t >= 0 ? texs[c.t] : V3{0.0f, 0.0f, 0.0f});
                }
                face.push_back(Corner{vi[c.v], ti[c.t], ni[c.n]});
            }
            of.push_back(face);
        }
        for (const auto &face : of) {
            for (size_t cur = 2; cur < face.size(); cur++) {
                const Corner tri[3] = {face[0], face[cur - 1], face[cur]};
                for (const Corner &c : tri) {
                    obj.xyz.insert(obj.xyz.end(), {ov[c.v].x, ov[c.v].y, ov[c.v].z});
                    obj.nrm.insert(obj.nrm.end(), {on[c.n].x, on[c.n].y, on[c.n].z});
                    obj.uv.insert(obj.uv.end(), {ot[c.t].x, ot[c.t].y, ot[c.t].z});
                }
            }
        }
        M->objects.push_back(std::move(obj));
    }
    *out = M;
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_obj_read");
}

int32_t dr_mesh_file_objects(const dr_mesh_file *m) { return m ? (int32_t)m->objects.size() : 0; }

const char *dr_mesh_file_object_name(const dr_mesh_file *m, int32_t i) {
    if (!m || i < 0 || i >= (int32_t)m->objects.size()) return nullptr;
    return m->objects[i].name.c_str();
}

int32_t dr_mesh_file_object_triangles(const dr_mesh_file *m, int32_t i) {
    if (!m || i < 0 || i >= (int32_t)m->objects.size()) return -1;
    return (int32_t)(m->objects[i].xyz.size() / 9);
}

dr_status dr_mesh_file_object_data(const dr_mesh_file *m, int32_t i, float *xyz, float *nrm, float *uv) try {
    if (!m || i < 0 || i >= (int32_t)m->objects.size()) return fail(DR_E_ARG, "dr_mesh_file_object_data: bad object");
    const auto &o = m->objects[i];
    if (xyz) std::memcpy(xyz, o.xyz.data(), o.xyz.size() * sizeof(float));
    if (nrm) std::memcpy(nrm, o.nrm.data(), o.nrm.size() * sizeof(float));
    if (uv) std::memcpy(uv, o.uv.data(), o.uv.size() * sizeof(float));
    return DR_OK;
} catch (...) {
    return dr_internal_exception("dr_mesh_file_object_data");
}

void dr_mesh_file_destroy(dr_mesh_file *m) { delete m; }

}  // extern "C"
