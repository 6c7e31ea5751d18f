// Scene ingest: the reference's scene JSON (src/util/Config.cpp:3-22), OBJ meshes
// (src/loader/OBJLoader.cpp:3-105), material JSON files (src/loader/MaterialLoader.cpp:9-36)
// and RGBE .hdr maps (src/loader/HDRLoader.cpp:5-152), assembled as Scene::add does
// (src/core/Scene.cpp:7-36).
//
// Arithmetic that decides vertex bits follows the reference step by step so that a scene
// loaded here equals the reference's: OBJ numbers are parsed straight to float (strtof, as
// libstdc++'s operator>> does), JSON numbers through double then cast to float (as the
// vendored JSON library stores them), per-object normalisation into [-1,1]
// (src/core/Object.cpp:40-83) and the S*T*R transform as 4x4 float matrices multiplied in
// the reference's loop order (include/math/LinearMath.h Mat4f::operator*, Transform.cpp:13-33).
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

#include <omp.h>

#include <algorithm>

#include "tt_internal.h"

namespace tt {

// ---- minimal JSON --------------------------------------------------------------------------
struct Json {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double num = 0.0;
    bool is_int = false;
    long long inum = 0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;  // sorted by key, like the reference's JSON objects

    const Json *find(const std::string &k) const {
        if (kind != OBJ) return nullptr;
        auto it = obj.find(k);
        return it == obj.end() ? nullptr : &it->second;
    }
    float as_float() const { return is_int ? (float)inum : (float)num; }
};

class JsonParser {
public:
    explicit JsonParser(const std::string &s) : s_(s) {}
    bool parse(Json &out, std::string &err) {
        pos_ = 0;
        if (!value(out)) {
            err = "JSON syntax error at byte " + std::to_string(pos_);
            return false;
        }
        ws();
        if (pos_ != s_.size()) {
            err = "trailing characters after JSON value at byte " + std::to_string(pos_);
            return false;
        }
        return true;
    }

private:
    const std::string &s_;
    size_t pos_ = 0;
    int depth_ = 0;

    void ws() {
        while (pos_ < s_.size() && (s_[pos_] == ' ' || s_[pos_] == '\t' || s_[pos_] == '\n' || s_[pos_] == '\r'))
            pos_++;
    }
    bool lit(const char *w) {
        size_t n = strlen(w);
        if (s_.compare(pos_, n, w) != 0) return false;
        pos_ += n;
        return true;
    }
    bool string(std::string &out) {
        if (pos_ >= s_.size() || s_[pos_] != '"') return false;
        pos_++;
        while (pos_ < s_.size() && s_[pos_] != '"') {
            char c = s_[pos_++];
            if (c == '\\') {
                if (pos_ >= s_.size()) return false;
                char e = s_[pos_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (pos_ + 4 > s_.size()) return false;
                        unsigned cp = (unsigned)strtoul(s_.substr(pos_, 4).c_str(), nullptr, 16);
                        pos_ += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 63)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 63));
                               out += (char)(0x80 | (cp & 63)); }
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (pos_ >= s_.size()) return false;
        pos_++;
        return true;
    }
    bool value(Json &v) {
        if (++depth_ > 256) return false;
        ws();
        bool ok = false;
        if (pos_ >= s_.size()) ok = false;
        else if (s_[pos_] == '{') {
            v.kind = Json::OBJ;
            pos_++;
            ws();
            if (pos_ < s_.size() && s_[pos_] == '}') { pos_++; ok = true; }
            else {
                while (true) {
                    ws();
                    std::string k;
                    if (!string(k)) break;
                    ws();
                    if (pos_ >= s_.size() || s_[pos_] != ':') break;
                    pos_++;
                    Json item;
                    if (!value(item)) break;
                    v.obj[k] = std::move(item);
                    ws();
                    if (pos_ < s_.size() && s_[pos_] == ',') { pos_++; continue; }
                    if (pos_ < s_.size() && s_[pos_] == '}') { pos_++; ok = true; }
                    break;
                }
            }
        } else if (s_[pos_] == '[') {
            v.kind = Json::ARR;
            pos_++;
            ws();
            if (pos_ < s_.size() && s_[pos_] == ']') { pos_++; ok = true; }
            else {
                while (true) {
                    Json item;
                    if (!value(item)) break;
                    v.arr.push_back(std::move(item));
                    ws();
                    if (pos_ < s_.size() && s_[pos_] == ',') { pos_++; continue; }
                    if (pos_ < s_.size() && s_[pos_] == ']') { pos_++; ok = true; }
                    break;
                }
            }
        } else if (s_[pos_] == '"') {
            v.kind = Json::STR;
            ok = string(v.str);
        } else if (lit("true")) { v.kind = Json::BOOL; v.b = true; ok = true; }
        else if (lit("false")) { v.kind = Json::BOOL; v.b = false; ok = true; }
        else if (lit("null")) { v.kind = Json::NUL; ok = true; }
        else {
            const char *start = s_.c_str() + pos_;
            char *end = nullptr;
            size_t n = 0;
            while (pos_ + n < s_.size() && strchr("+-0123456789.eE", s_[pos_ + n])) n++;
            std::string tok = s_.substr(pos_, n);
            if (n > 0) {
                bool integral = tok.find_first_of(".eE") == std::string::npos;
                v.kind = Json::NUM;
                if (integral) {
                    errno = 0;
                    v.inum = strtoll(tok.c_str(), &end, 10);
                    v.is_int = errno == 0 && end && *end == 0;
                    v.num = (double)v.inum;
                }
                if (!v.is_int) {
                    v.num = strtod(tok.c_str(), &end);
                    if (!end || *end != 0) n = 0;
                }
            }
            (void)start;
            ok = n > 0;
            pos_ += n;
        }
        depth_--;
        return ok;
    }
};

static bool read_file(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f.good()) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

static tt_status parse_json_file(const std::string &path, Json &out) {
    std::string text;
    if (!read_file(path, text)) return fail(TT_ERR_IO, "cannot read " + path);
    std::string err;
    if (!JsonParser(text).parse(out, err)) return fail(TT_ERR_FORMAT, path + ": " + err);
    return TT_OK;
}

static bool json_vec3(const Json *j, V3 &out) {
    if (!j || j->kind != Json::ARR || j->arr.size() < 3) return false;
    for (int i = 0; i < 3; i++)
        if (j->arr[i].kind != Json::NUM) return false;
    out = V3(j->arr[0].as_float(), j->arr[1].as_float(), j->arr[2].as_float());
    return true;
}

// ---- 4x4 float matrices, in the reference's arithmetic order --------------------------------
struct M4 {
    float m[4][4];
    static M4 identity() {
        M4 r;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) r.m[i][j] = i == j ? 1.0f : 0.0f;
        return r;
    }
    M4 operator*(const M4 &b) const {
        M4 r;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                r.m[i][j] = 0;
                for (int k = 0; k < 4; k++) r.m[i][j] += m[i][k] * b.m[k][j];
            }
        return r;
    }
    // Mat4f * Vec4f: each row dotted with v, accumulated from 0 in index order.
    void apply(const float v[4], float out[4]) const {
        for (int i = 0; i < 4; i++) {
            float s = 0;
            for (int k = 0; k < 4; k++) s += m[i][k] * v[k];
            out[i] = s;
        }
    }
};

static M4 row_matrix(const float rows[4][4]) {
    M4 r;
    memcpy(r.m, rows, sizeof(r.m));
    return r;
}

// Transform(geometryJson) (src/geometry/Transform.cpp:13-33): I * S * T * R, with
// R = rotY(y) * rotX(x) * rotZ(z) from degrees (include/math/PoseMath.h:24-57).
static M4 transform_matrix(const Json &geom) {
    M4 m = M4::identity();
    const Json *t = geom.find("transform");
    if (!t || t->kind != Json::OBJ) return m;
    V3 v;
    if (json_vec3(t->find("scale"), v)) {
        const float r[4][4] = {{v.x, 0, 0, 0}, {0, v.y, 0, 0}, {0, 0, v.z, 0}, {0, 0, 0, 1}};
        m = m * row_matrix(r);
    }
    if (json_vec3(t->find("translate"), v)) {
        const float r[4][4] = {{1, 0, 0, v.x}, {0, 1, 0, v.y}, {0, 0, 1, v.z}, {0, 0, 0, 1}};
        m = m * row_matrix(r);
    }
    if (json_vec3(t->find("orientation"), v)) {
        V3 a = (v / 180.0f) * (float)M_PI;
        const float ry[4][4] = {{cosf(a.y), 0, sinf(a.y), 0}, {0, 1, 0, 0}, {-sinf(a.y), 0, cosf(a.y), 0}, {0, 0, 0, 1}};
        const float rx[4][4] = {{1, 0, 0, 0}, {0, cosf(a.x), -sinf(a.x), 0}, {0, sinf(a.x), cosf(a.x), 0}, {0, 0, 0, 1}};
        const float rz[4][4] = {{cosf(a.z), -sinf(a.z), 0, 0}, {sinf(a.z), cosf(a.z), 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
        m = m * (row_matrix(ry) * row_matrix(rx) * row_matrix(rz));
    }
    return m;
}

// ---- materials -------------------------------------------------------------------------
static tt_status parse_material(const std::string &name, const Json &j, MaterialRec &out) {
    memset(&out, 0, sizeof(out));
    out.ior = 1.5f;
    const Json *type = j.find("type");
    if (!type || type->kind != Json::STR) return fail(TT_ERR_FORMAT, "material " + name + " has no type");
    V3 v;
    if (json_vec3(j.find("emission"), v)) { out.emission[0] = v.x; out.emission[1] = v.y; out.emission[2] = v.z; }
    auto color = [&](const char *key, float *dst) -> bool {
        V3 c;
        if (!json_vec3(j.find(key), c)) return false;
        dst[0] = c.x; dst[1] = c.y; dst[2] = c.z;
        return true;
    };
    const std::string &t = type->str;
    if (t == "Diff") { out.kind = MAT_DIFF; if (!color("diffuseColor", out.color)) goto missing; }
    else if (t == "Metal") { out.kind = MAT_METAL; if (!color("color", out.color)) goto missing; }
    else if (t == "Spec") { out.kind = MAT_SPEC; if (!color("color", out.color)) goto missing; }
    else if (t == "Refr") { out.kind = MAT_REFR; out.ior = 1.4f; }
    else if (t == "Coat") {
        out.kind = MAT_COAT;
        if (!color("diffuseColor", out.color) || !color("specularColor", out.color2)) goto missing;
    } else if (t == "GGX") {
        out.kind = MAT_GGX;
        if (!color("F0", out.color) && !color("color", out.color)) goto missing;
        const Json *r = j.find("roughness");
        out.roughness = (r && r->kind == Json::NUM) ? r->as_float() : 0.5f;
    } else if (t == "Dielectric") {
        out.kind = MAT_DIELECTRIC;
        const Json *r = j.find("ior");
        out.ior = (r && r->kind == Json::NUM) ? r->as_float() : 1.5f;
    } else {
        return fail(TT_ERR_FORMAT, "material " + name + " has unknown type " + t);
    }
    return TT_OK;
missing:
    return fail(TT_ERR_FORMAT, "material " + name + " misses its colour");
}

// MaterialLoader::load + Scene::add(MaterialPool*): materials take consecutive scene indices
// in key order (the pool is a std::map, src/material/MaterialPool.cpp:12-24).
static tt_status load_material_pool(const std::string &path, Scene &sc, std::map<std::string, int32_t> &pool) {
    Json j;
    tt_status st = parse_json_file(path, j);
    if (st != TT_OK) return st;
    if (j.kind != Json::OBJ) return fail(TT_ERR_FORMAT, path + ": material file is not a JSON object");
    for (auto &kv : j.obj) {
        MaterialRec m;
        if ((st = parse_material(kv.first, kv.second, m)) != TT_OK) return st;
        pool[kv.first] = (int32_t)sc.materials.size();
        sc.materials.push_back(m);
        sc.material_names.push_back(kv.first);
    }
    return TT_OK;
}

// ---- OBJ ---------------------------------------------------------------------------------
struct ObjGroup {
    std::vector<int32_t> v, n;  // 3 per triangle
    int32_t mat = -1;
};

static bool next_float(const char *&p, float &out) {
    while (*p == ' ' || *p == '\t' || *p == '\r') p++;
    if (!*p) return false;
    char *end = nullptr;
    out = strtof(p, &end);
    if (end == p) return false;
    p = end;
    return true;
}

// One line-aligned chunk of an OBJ file, parsed on its own: vertices, normals, triangles (fan
// triangulation, 0-based indices) and the group / material statements in file order, each with
// the number of this chunk's triangles that precede it.
struct ObjEvent {
    int kind;        // 0 "g", 1 "usemtl", 2 "mtllib"
    size_t tri;
    std::string name;
};
struct ObjChunk {
    std::vector<V3> v, vn;
    std::vector<int32_t> fv, fn;  // 3 per triangle
    std::vector<ObjEvent> ev;
    std::string error;  // the first malformed line of the chunk (parsing stopped there)
};

// Parses the NUL-separated lines in [b, e); every line ends in '\0' or at e, and *e == '\0'.
static void parse_obj_chunk(char *b, char *e, const std::string &file, ObjChunk &c) {
    for (char *line = b; line < e;) {
        char *nl = static_cast<char *>(memchr(line, '\n', (size_t)(e - line)));
        char *stop = nl ? nl : e;
        *stop = '\0';
        const char *p = line;
        line = stop + 1;
        while (*p == ' ' || *p == '\t') p++;
        const char *k = p;
        while (*p && *p != ' ' && *p != '\t' && *p != '\r') p++;
        const size_t klen = (size_t)(p - k);
        while (*p == ' ' || *p == '\t') p++;
        auto key_is = [&](const char *w) { return strlen(w) == klen && strncmp(k, w, klen) == 0; };
        auto first_word = [&]() {
            const char *q = p;
            while (*q && *q != ' ' && *q != '\t' && *q != '\r') q++;
            return std::string(p, q);
        };
        if (key_is("g")) {
            c.ev.push_back({0, c.fv.size() / 3, std::string()});
        } else if (key_is("mtllib")) {
            c.ev.push_back({2, c.fv.size() / 3, first_word()});
        } else if (key_is("usemtl")) {
            c.ev.push_back({1, c.fv.size() / 3, first_word()});
        } else if (key_is("v") || key_is("vn")) {
            std::vector<V3> &dst = klen == 1 ? c.v : c.vn;
            const char *q = p;
            float x, y, z;
            while (next_float(q, x)) {
                if (!next_float(q, y) || !next_float(q, z)) {
                    c.error = file + ": short " + std::string(k, klen) + " line";
                    return;
                }
                dst.push_back(V3(x, y, z));
            }
        } else if (key_is("f")) {
            int fv[64], fn[64], cnt = 0;
            int v = 1, n = 1;
            const char *q = p;
            while (*q && cnt < 64) {
                char *endp = nullptr;
                long a = strtol(q, &endp, 10);
                if (endp == q) break;
                v = (int)a;
                q = endp;
                if (*q == '/') {
                    q++;
                    if (*q == '/') {
                        q++;
                        n = (int)strtol(q, &endp, 10);
                        q = endp;
                    } else {
                        strtol(q, &endp, 10);  // texture index: unused
                        q = endp;
                        if (*q == '/') {
                            q++;
                            n = (int)strtol(q, &endp, 10);
                            q = endp;
                        }
                    }
                }
                fv[cnt] = v - 1;
                fn[cnt] = n - 1;
                cnt++;
                while (*q == ' ' || *q == '\t' || *q == '\r') q++;
            }
            if (*q && cnt == 64) {
                c.error = file + ": face with more than 64 vertices";
                return;
            }
            for (int i = 0; i + 2 < cnt; i++) {
                c.fv.insert(c.fv.end(), {fv[0], fv[i + 1], fv[i + 2]});
                c.fn.insert(c.fn.end(), {fn[0], fn[i + 1], fn[i + 2]});
            }
        }
    }
}

// OBJLoader::load + Object::postProcess + Object::apply + Scene::add(Object*), the file parsed in
// line-aligned chunks on all host threads and the chunks' statements replayed in file order, so
// the result is that of one sequential pass. Beyond the reference: an OBJ without `vn` lines gets
// area-weighted vertex normals, and when the normal and vertex counts differ both arrays are
// transformed in full (the reference indexes normals with the vertex loop, reading past the end
// of a shorter normal array and leaving the extra normals of a longer one untransformed).
static tt_status load_obj(const std::string &file, const M4 &xf, Scene &sc) {
    std::vector<char> buf;
    {
        FILE *f = fopen(file.c_str(), "rb");
        if (!f) return fail(TT_ERR_IO, "cannot read OBJ " + file);
        std::fseek(f, 0, SEEK_END);
        const long size = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (size < 0) {
            fclose(f);
            return fail(TT_ERR_IO, "cannot read OBJ " + file);
        }
        buf.resize((size_t)size + 1);
        const size_t got = size ? fread(buf.data(), 1, (size_t)size, f) : 0;
        fclose(f);
        if (got != (size_t)size) return fail(TT_ERR_IO, "short read of OBJ " + file);
        buf[(size_t)size] = '\0';
    }
    const size_t size = buf.size() - 1;
    const int nchunks = std::max(1, omp_get_max_threads());
    std::vector<size_t> cut(nchunks + 1, size);
    cut[0] = 0;
    for (int i = 1; i < nchunks; i++) {
        size_t c = std::max(cut[i - 1], size / nchunks * i);
        while (c < size && c > 0 && buf[c - 1] != '\n') c++;  // start each chunk at a line start
        cut[i] = c;
    }
    std::vector<ObjChunk> chunks(nchunks);
#pragma omp parallel for schedule(static, 1)
    for (int i = 0; i < nchunks; i++) {
        if (cut[i] < cut[i + 1]) {
            char *b = buf.data() + cut[i], *e = buf.data() + cut[i + 1];
            // the chunk's last byte is its last line's '\n' (or the file ends there): that line ends
            // at a terminator the chunk owns, and the splitter writes only inside [b, e]
            const char saved = *(e - 1);
            if (saved == '\n') *(e - 1) = '\0';
            parse_obj_chunk(b, saved == '\n' ? e - 1 : e, file, chunks[i]);
        }
    }
    std::vector<V3> verts, norms;
    std::vector<ObjGroup> groups;
    std::map<std::string, int32_t> pool;
    bool have_pool = false;
    auto add_tris = [&](const ObjChunk &c, size_t t0, size_t t1) {
        if (t1 <= t0) return;
        if (groups.empty()) groups.emplace_back();
        ObjGroup &g = groups.back();
        g.v.insert(g.v.end(), c.fv.begin() + 3 * t0, c.fv.begin() + 3 * t1);
        g.n.insert(g.n.end(), c.fn.begin() + 3 * t0, c.fn.begin() + 3 * t1);
    };
    for (const ObjChunk &c : chunks) {
        size_t t = 0;
        for (const ObjEvent &ev : c.ev) {
            add_tris(c, t, ev.tri);
            t = ev.tri;
            if (ev.kind == 0) {
                groups.emplace_back();
            } else if (ev.kind == 2) {
                std::string prefix;
                size_t slash = file.find_last_of('/');
                if (slash != std::string::npos) prefix = file.substr(0, slash + 1);
                tt_status st = load_material_pool(prefix + ev.name, sc, pool);
                if (st != TT_OK) return st;
                have_pool = true;
            } else {
                if (!have_pool) return fail(TT_ERR_FORMAT, file + ": usemtl before mtllib");
                auto it = pool.find(ev.name);
                if (it == pool.end()) return fail(TT_ERR_FORMAT, "Material " + ev.name + " not found");
                if (groups.empty()) groups.emplace_back();
                groups.back().mat = it->second;
            }
        }
        add_tris(c, t, c.fv.size() / 3);
        verts.insert(verts.end(), c.v.begin(), c.v.end());
        norms.insert(norms.end(), c.vn.begin(), c.vn.end());
        if (!c.error.empty()) return fail(TT_ERR_FORMAT, c.error);
    }
    if (!have_pool) return fail(TT_ERR_FORMAT, file + ": OBJ has no mtllib (the scene needs its material pool)");
    for (const ObjGroup &g : groups) {
        if (!g.v.empty() && g.mat < 0) return fail(TT_ERR_FORMAT, file + ": group without usemtl");
        for (int32_t i : g.v)
            if (i < 0 || (size_t)i >= verts.size()) return fail(TT_ERR_FORMAT, file + ": face vertex out of range");
    }
    if (norms.empty()) {
        // no normals in the file: area-weighted vertex normals, indexed like the vertices
        norms.assign(verts.size(), V3(0.0f, 0.0f, 0.0f));
        for (ObjGroup &g : groups) {
            for (size_t t = 0; t + 2 < g.v.size(); t += 3) {
                const V3 &a0 = verts[g.v[t]], &a1 = verts[g.v[t + 1]], &a2 = verts[g.v[t + 2]];
                const V3 fnrm = cross3(a1 - a0, a2 - a0);
                for (int k = 0; k < 3; k++) norms[g.v[t + k]] = norms[g.v[t + k]] + fnrm;
            }
            g.n = g.v;
        }
        for (V3 &n : norms)
            if (!(dot3(n, n) > 0.0f)) n = V3(0.0f, 1.0f, 0.0f);
    }
    for (const ObjGroup &g : groups)
        for (int32_t i : g.n)
            if (i < 0 || (size_t)i >= norms.size()) return fail(TT_ERR_FORMAT, file + ": face normal out of range");

    // Object::postProcess: centre the face-referenced bounds at the origin, scale into [-1,1].
    V3 minp(FLT_MAX, FLT_MAX, FLT_MAX), maxp(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    for (const ObjGroup &g : groups)
        for (int32_t i : g.v) {
            minp = vmin3(minp, verts[i]);
            maxp = vmax3(maxp, verts[i]);
        }
    V3 c((maxp.x + minp.x) * 0.5f, (maxp.y + minp.y) * 0.5f, (maxp.z + minp.z) * 0.5f);
    minp = minp - c;
    maxp = maxp - c;
    float maxi = 0;
    for (float a : {minp.x, minp.y, minp.z, maxp.x, maxp.y, maxp.z}) maxi = std::max(maxi, std::fabs(a));
    float scale = 1.0f / maxi;
    for (V3 &v : verts) {
        v = v - c;
        v = v * scale;
    }
    // Object::apply(Transform): vertices with w = 1, normals with w = 0 then normalised (the
    // reference's loop over the vertex count when the counts agree, each array in full otherwise)
    const size_t nn = norms.size() == verts.size() ? verts.size() : norms.size();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)std::max(verts.size(), nn); i++) {
        float out[4];
        if ((size_t)i < verts.size()) {
            float in[4] = {verts[i].x, verts[i].y, verts[i].z, 1.0f};
            xf.apply(in, out);
            verts[i] = V3(out[0], out[1], out[2]);
        }
        if ((size_t)i < nn) {
            float nin[4] = {norms[i].x, norms[i].y, norms[i].z, 0.0f};
            xf.apply(nin, out);
            norms[i] = normalized(V3(out[0], out[1], out[2]));
        }
    }
    // Scene::add(Object*)
    const int32_t vbase = (int32_t)sc.vertices.size(), nbase = (int32_t)sc.normals.size();
    sc.vertices.insert(sc.vertices.end(), verts.begin(), verts.end());
    sc.normals.insert(sc.normals.end(), norms.begin(), norms.end());
    for (const ObjGroup &g : groups) {
        for (size_t t = 0; t < g.v.size() / 3; t++) {
            for (int k = 0; k < 3; k++) {
                sc.vidx.push_back(g.v[3 * t + k] + vbase);
                sc.nidx.push_back(g.n[3 * t + k] + nbase);
            }
            sc.mat.push_back((uint32_t)g.mat);
        }
    }
    return TT_OK;
}

// ---- RGBE .hdr ------------------------------------------------------------------------------
// A Radiance picture (src/loader/HDRLoader.cpp reads the same files): "#?RADIANCE", header lines
// up to an empty line, a "-Y <height> +X <width>" line, then `height` scanlines of `width` RGBE
// pixels (8-bit mantissas sharing an exponent biased by 128). A scanline is stored in one of two
// codings:
//   flat            4-byte R,G,B,E pixels. A pixel (1, 1, 1, n) stands for n copies of the pixel
//                   before it; each repeat pixel that directly follows another multiplies its
//                   count by 256 (the older run-length form of the format).
//   adaptive RLE    widths 8..32767 only: the bytes 2, 2, width >> 8, width & 255, then the R, G, B
//                   and E components one after another, each as packets: a count byte c > 128 is
//                   followed by one byte repeated c - 128 times, any other c by c literal bytes.
// The decoder works on the file's bytes in memory. A scanline that runs past the end of the data
// ends the picture; it and the rows after it stay zero.
namespace {

struct ByteCursor {
    const unsigned char *p, *end;
    bool overrun = false;
    size_t left() const { return (size_t)(end - p); }
    // the next byte, or 0 (recorded as an overrun) past the end
    unsigned char take() {
        if (p < end) return *p++;
        overrun = true;
        return 0;
    }
};

enum class ScanlineCoding { Flat, AdaptiveRle };

ScanlineCoding scanline_coding(const ByteCursor &in, long width) {
    if (width < 8 || width > 0x7fff || in.left() < 4) return ScanlineCoding::Flat;
    // a flat scanline cannot start with these bytes unless its first pixel has a 2,2 red/green
    // mantissa pair and a blue mantissa below 128, which the format reserves for the RLE marker
    return (in.p[0] == 2 && in.p[1] == 2 && (in.p[2] & 0x80) == 0) ? ScanlineCoding::AdaptiveRle
                                                                  : ScanlineCoding::Flat;
}

// One scanline into `px` (width x 4 bytes). Returns false when the data ends inside it.
bool decode_scanline(ByteCursor &in, long width, unsigned char *px) {
    if (scanline_coding(in, width) == ScanlineCoding::AdaptiveRle) {
        in.p += 4;  // 2, 2 and the width, which the pixel count already gives
        for (int comp = 0; comp < 4; comp++) {
            long x = 0;
            while (x < width) {
                if (!in.left()) return false;
                const int count = in.take();
                if (count > 128) {
                    const unsigned char value = in.take();
                    for (int k = count - 128; k > 0 && x < width; k--) px[4 * x++ + comp] = value;
                } else {
                    for (int k = count; k > 0 && x < width; k--) px[4 * x++ + comp] = in.take();
                }
            }
        }
        return !in.overrun;
    }
    unsigned char prev[4] = {0, 0, 0, 0};  // the pixel a repeat at the start of a scanline copies
    int shift = 0;
    long x = 0;
    while (x < width) {
        if (in.left() < 4) return false;
        const unsigned char *q = in.p;
        in.p += 4;
        if (q[0] == 1 && q[1] == 1 && q[2] == 1) {
            long repeat = shift < 32 ? (long)q[3] << shift : (q[3] ? width : 0);
            for (; repeat > 0 && x < width; repeat--, x++) memcpy(px + 4 * x, prev, 4);
            shift += 8;
        } else {
            memcpy(px + 4 * x, q, 4);
            memcpy(prev, q, 4);
            x++;
            shift = 0;
        }
    }
    return true;
}

}  // namespace

tt_status load_hdr(const std::string &path, int32_t &w_out, int32_t &h_out, std::vector<float> &rgb) {
    std::vector<unsigned char> bytes;
    {
        FILE *f = fopen(path.c_str(), "rb");
        if (!f) return fail(TT_ERR_IO, "HDR environment map not found: " + path);
        unsigned char chunk[1 << 16];
        size_t got;
        while ((got = fread(chunk, 1, sizeof(chunk), f)) > 0) bytes.insert(bytes.end(), chunk, chunk + got);
        fclose(f);
    }
    ByteCursor in{bytes.data(), bytes.data() + bytes.size()};
    if (in.left() < 11 || memcmp(in.p, "#?RADIANCE", 10) != 0)
        return fail(TT_ERR_FORMAT, path + ": not a RADIANCE file");
    in.p += 11;  // the magic and the byte after it
    // header lines end at an empty line
    for (unsigned char prev = 0;;) {
        if (!in.left()) return fail(TT_ERR_FORMAT, path + ": header not terminated");
        const unsigned char c = in.take();
        if (c == '\n' && prev == '\n') break;
        prev = c;
    }
    std::string reso;
    while (in.left() && reso.size() < 255) {
        const char c = (char)in.take();
        reso.push_back(c);
        if (c == '\n') break;
    }
    long w = 0, h = 0;
    if (sscanf(reso.c_str(), "-Y %ld +X %ld", &h, &w) != 2 || w <= 0 || h <= 0 || w * h > (1L << 28))
        return fail(TT_ERR_FORMAT, path + ": bad resolution line");
    rgb.assign((size_t)w * h * 3, 0.0f);
    std::vector<unsigned char> px((size_t)w * 4);
    for (long y = 0; y < h; y++) {
        if (!decode_scanline(in, w, px.data())) break;
        float *dst = rgb.data() + (size_t)y * w * 3;
        for (long x = 0; x < w; x++) {
            const float scale = ldexpf(1.0f, (int)px[4 * x + 3] - 128);
            for (int c = 0; c < 3; c++) dst[3 * x + c] = (px[4 * x + c] / 256.0f) * scale;
        }
    }
    w_out = (int32_t)w;
    h_out = (int32_t)h;
    return TT_OK;
}

// ---- scene JSON -------------------------------------------------------------------------------
static std::string resolve(const std::string &base_dir, const std::string &p) {
    if (p.empty() || p[0] == '/') return p;
    std::ifstream probe(p);
    if (probe.good()) return p;  // relative to the working directory, as the reference reads it
    return base_dir + p;
}

tt_status load_scene_json(const std::string &path, Scene &sc) {
    Json cfg;
    tt_status st = parse_json_file(path, cfg);
    if (st != TT_OK) return st;
    std::string base_dir;
    size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) base_dir = path.substr(0, slash + 1);
    auto req = [&](const char *k, Json::Kind kind) -> const Json * {
        const Json *j = cfg.find(k);
        return (j && j->kind == kind) ? j : nullptr;
    };
    const Json *camera = req("camera", Json::OBJ);
    const Json *workdir = req("work-dir", Json::STR);
    const Json *hdr = req("hdr-file-name", Json::STR);
    const Json *mtl = req("material-file", Json::STR);
    const Json *samples = req("samples", Json::NUM);
    const Json *objects = req("objects", Json::ARR);
    if (!camera || !workdir || !hdr || !mtl || !samples || !objects)
        return fail(TT_ERR_FORMAT, path + ": missing one of camera, work-dir, hdr-file-name, material-file, samples, objects");
    const Json *w = camera->find("width"), *h = camera->find("height");
    if (!w || !h || w->kind != Json::NUM || h->kind != Json::NUM) return fail(TT_ERR_FORMAT, path + ": camera width/height");
    sc = Scene();
    sc.work_dir = workdir->str;
    sc.hdr_file = resolve(base_dir, hdr->str);
    sc.material_file = resolve(base_dir, mtl->str);
    sc.samples = (int32_t)samples->inum;
    if (const Json *b = cfg.find("bvh-reload")) sc.bvh_reload = b->b;
    if (const Json *b = cfg.find("material-reload")) sc.material_reload = b->b;
    if (const Json *d = cfg.find("max-depth")) sc.max_depth = (int32_t)d->inum;
    if (const Json *d = cfg.find("rr-depth")) sc.rr_depth = (int32_t)d->inum;
    CameraConfig &cam = sc.camera;
    cam.width = (int32_t)w->inum;
    cam.height = (int32_t)h->inum;
    V3 v;
    if (json_vec3(camera->find("position"), v)) cam.position = v;
    if (const Json *j = camera->find("yaw")) cam.yaw = j->as_float();
    if (const Json *j = camera->find("pitch")) cam.pitch = j->as_float();
    if (const Json *j = camera->find("focal")) cam.focal = j->as_float();
    if (const Json *j = camera->find("aperture")) cam.aperture = j->as_float();

    std::map<std::string, int32_t> master;
    if ((st = load_material_pool(sc.material_file, sc, master)) != TT_OK) return st;
    for (const Json &obj : objects->arr) {
        const Json *type = obj.find("type");
        if (!type || type->kind != Json::STR) return fail(TT_ERR_FORMAT, path + ": object without type");
        if (type->str == "Mesh") {
            const Json *file = obj.find("file");
            if (!file || file->kind != Json::STR) return fail(TT_ERR_FORMAT, path + ": Mesh without file");
            if ((st = load_obj(resolve(base_dir, file->str), transform_matrix(obj), sc)) != TT_OK) return st;
        } else if (type->str == "Plane" || type->str == "Sphere") {
            GeomRec g;
            memset(&g, 0, sizeof(g));
            const Json *m = obj.find("material");
            if (!m || m->kind != Json::STR || !master.count(m->str))
                return fail(TT_ERR_FORMAT, path + ": object material missing from the material file");
            g.mat = master[m->str];
            if (type->str == "Plane") {
                g.kind = GEOM_PLANE;
                V3 a, b, c;
                if (!json_vec3(obj.find("p0"), a) || !json_vec3(obj.find("p1"), b) || !json_vec3(obj.find("p2"), c))
                    return fail(TT_ERR_FORMAT, path + ": Plane needs p0, p1, p2");
                memcpy(g.p0, &a, 12);
                memcpy(g.p1, &b, 12);
                memcpy(g.p2, &c, 12);
            } else {
                g.kind = GEOM_SPHERE;
                const Json *r = obj.find("radius");
                if (!r || r->kind != Json::NUM || !json_vec3(obj.find("position"), v))
                    return fail(TT_ERR_FORMAT, path + ": Sphere needs radius and position");
                g.radius = r->as_float();
                memcpy(g.p0, &v, 12);
            }
            sc.geoms.push_back(g);
        }
        // other types are ignored, as in the reference
    }
    // An empty hdr-file-name means "no environment" (black on miss); a named file must load,
    // as HDRLoader::load throws when it is missing (src/loader/HDRLoader.cpp:11-17).
    if (!hdr->str.empty()) {
        if ((st = load_hdr(sc.hdr_file, sc.env_w, sc.env_h, sc.env_rgb)) != TT_OK) return st;
    }
    return TT_OK;
}

}  // namespace tt
