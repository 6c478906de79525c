// Scene ingestion for the C ABI (host code): the PLY reader of
// src/io/ply.cpp (read_ply: element `vertex` with x y z, element `face` with
// a 3-index list -> triangles, element `tet` with a 4-index list ->
// tetrahedra; ascii, binary_little_endian, binary_big_endian; positions kept
// as float like the reference's geometry_t) and the JSON scene loader of
// src/io/load_scene.cpp:83-365 (environment triangle meshes and soft
// tetrahedral objects, each optionally rescaled into its "box" and moved by
// its "translation").  Lights, colours and rendering options are read past.
#include <stdint.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sbs_gpu.h"

namespace {

struct PlyProperty {
    std::string name, type, count_type;  // count_type non-empty for lists
};
struct PlyElement {
    std::string name;
    uint64_t count = 0;
    std::vector<PlyProperty> props;
};

struct PlyData {
    std::vector<float> positions;
    std::vector<uint32_t> tris, tets;
};

int type_size(const std::string& t) {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
}

// One binary scalar of type t, as double; `swap` for big-endian files on a
// little-endian host (or the reverse).
bool read_binary(std::istream& is, const std::string& t, bool swap, double& out) {
    const int n = type_size(t);
    if (n == 0) return false;
    unsigned char b[8];
    if (!is.read(reinterpret_cast<char*>(b), n)) return false;
    if (swap)
        for (int i = 0; i < n / 2; ++i) std::swap(b[i], b[n - 1 - i]);
    if (t == "char" || t == "int8") out = (double)(int8_t)b[0];
    else if (t == "uchar" || t == "uint8") out = (double)b[0];
    else if (t == "short" || t == "int16") { int16_t v; std::memcpy(&v, b, 2); out = v; }
    else if (t == "ushort" || t == "uint16") { uint16_t v; std::memcpy(&v, b, 2); out = v; }
    else if (t == "int" || t == "int32") { int32_t v; std::memcpy(&v, b, 4); out = v; }
    else if (t == "uint" || t == "uint32") { uint32_t v; std::memcpy(&v, b, 4); out = v; }
    else if (t == "float" || t == "float32") { float v; std::memcpy(&v, b, 4); out = v; }
    else { double v; std::memcpy(&v, b, 8); out = v; }
    return true;
}

bool host_little_endian() {
    const uint16_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

// Parses a PLY file into positions, triangles and tets.  Returns false with
// a message on malformed input.
bool read_ply(const std::string& path, PlyData& out, std::string& err) {
    std::ifstream is(path, std::ios::binary);
    if (!is) { err = "cannot open " + path; return false; }
    std::string line;
    if (!std::getline(is, line) || line.compare(0, 3, "ply") != 0) { err = "not a PLY file"; return false; }
    std::string format;
    std::vector<PlyElement> elements;
    while (std::getline(is, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ls(line);
        std::string kw;
        ls >> kw;
        if (kw == "format") ls >> format;
        else if (kw == "element") {
            PlyElement e;
            ls >> e.name >> e.count;
            elements.push_back(e);
        } else if (kw == "property") {
            if (elements.empty()) { err = "property before element"; return false; }
            PlyProperty p;
            std::string t;
            ls >> t;
            if (t == "list") ls >> p.count_type >> p.type >> p.name;
            else { p.type = t; ls >> p.name; }
            elements.back().props.push_back(p);
        } else if (kw == "end_header") break;
    }
    const bool ascii = format == "ascii";
    const bool binary = format == "binary_little_endian" || format == "binary_big_endian";
    if (!ascii && !binary) { err = "unknown PLY format " + format; return false; }
    const bool swap = binary && ((format == "binary_little_endian") != host_little_endian());
    for (const PlyElement& e : elements) {
        const bool vert = e.name == "vertex", face = e.name == "face", tet = e.name == "tet";
        int ix = -1, iy = -1, iz = -1;
        for (size_t k = 0; k < e.props.size(); ++k) {
            if (e.props[k].name == "x") ix = (int)k;
            if (e.props[k].name == "y") iy = (int)k;
            if (e.props[k].name == "z") iz = (int)k;
        }
        for (uint64_t r = 0; r < e.count; ++r) {
            std::vector<double> scalars(e.props.size(), 0.0);
            std::vector<uint32_t> list;
            if (ascii) {
                if (!std::getline(is, line)) { err = "truncated PLY body"; return false; }
                std::istringstream ls(line);
                for (size_t k = 0; k < e.props.size(); ++k) {
                    std::string tok;
                    if (!e.props[k].count_type.empty()) {
                        long c;
                        if (!(ls >> c) || c < 0 || c > 64) { err = "bad PLY list"; return false; }
                        for (long i = 0; i < c; ++i) {
                            long v;
                            if (!(ls >> v) || v < 0) { err = "bad PLY list"; return false; }
                            list.push_back((uint32_t)v);
                        }
                    } else if (!(ls >> tok)) {
                        err = "bad PLY value";
                        return false;
                    } else {
                        // the reference parses values with std::stof
                        scalars[k] = (double)std::strtof(tok.c_str(), nullptr);
                    }
                }
            } else {
                for (size_t k = 0; k < e.props.size(); ++k) {
                    if (!e.props[k].count_type.empty()) {
                        double c;
                        if (!read_binary(is, e.props[k].count_type, swap, c) || c < 0 || c > 64) {
                            err = "bad PLY list";
                            return false;
                        }
                        for (int i = 0; i < (int)c; ++i) {
                            double v;
                            if (!read_binary(is, e.props[k].type, swap, v) || v < 0) { err = "bad PLY list"; return false; }
                            list.push_back((uint32_t)v);
                        }
                    } else if (!read_binary(is, e.props[k].type, swap, scalars[k])) {
                        err = "truncated PLY body";
                        return false;
                    }
                }
            }
            if (vert) {
                if (ix < 0 || iy < 0 || iz < 0) { err = "vertex without x y z"; return false; }
                out.positions.push_back((float)scalars[ix]);
                out.positions.push_back((float)scalars[iy]);
                out.positions.push_back((float)scalars[iz]);
            } else if (face) {
                if (list.size() != 3) { err = "only triangle faces are read"; return false; }
                out.tris.insert(out.tris.end(), list.begin(), list.end());
            } else if (tet) {
                if (list.size() != 4) { err = "tet element without 4 indices"; return false; }
                out.tets.insert(out.tets.end(), list.begin(), list.end());
            }
        }
    }
    const uint64_t nv = out.positions.size() / 3;
    for (uint32_t i : out.tris)
        if (i >= nv) { err = "face index out of range"; return false; }
    for (uint32_t i : out.tets)
        if (i >= nv) { err = "tet index out of range"; return false; }
    return true;
}

}  // namespace

extern "C" sbs_status sbs_io_read_ply(const char* path, float* positions, uint32_t cap_verts, uint32_t* n_verts,
                                      uint32_t* tris, uint32_t cap_tris, uint32_t* n_tris, uint32_t* tets,
                                      uint32_t cap_tets, uint32_t* n_tets) {
    if (!path) return SBS_EINVAL;
    PlyData d;
    std::string err;
    if (!read_ply(path, d, err)) return SBS_EINVAL;
    const uint32_t nv = (uint32_t)(d.positions.size() / 3), nf = (uint32_t)(d.tris.size() / 3),
                   nt = (uint32_t)(d.tets.size() / 4);
    if (n_verts) *n_verts = nv;
    if (n_tris) *n_tris = nf;
    if (n_tets) *n_tets = nt;
    if (positions) {
        if (cap_verts < nv) return SBS_EINVAL;
        std::memcpy(positions, d.positions.data(), d.positions.size() * sizeof(float));
    }
    if (tris) {
        if (cap_tris < nf) return SBS_EINVAL;
        std::memcpy(tris, d.tris.data(), d.tris.size() * sizeof(uint32_t));
    }
    if (tets) {
        if (cap_tets < nt) return SBS_EINVAL;
        std::memcpy(tets, d.tets.data(), d.tets.size() * sizeof(uint32_t));
    }
    return SBS_OK;
}

namespace {

// Minimal JSON (RFC 8259) reader: objects, arrays, strings (with escapes),
// numbers, true/false/null.
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    const JVal* get(const char* key) const {
        if (kind != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    double number(const char* key, double def) const {
        const JVal* v = get(key);
        return v && v->kind == Num ? v->num : def;
    }
};

struct JParser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit JParser(const std::string& text) : s(text) {}
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    bool lit(const char* w) {
        const size_t n = std::strlen(w);
        if (s.compare(i, n, w) != 0) return false;
        i += n;
        return true;
    }
    bool string(std::string& out) {
        if (i >= s.size() || s[i] != '"') return false;
        ++i;
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) return false;
                const char e = s[i++];
                if (e == 'n') c = '\n';
                else if (e == 't') c = '\t';
                else if (e == 'r') c = '\r';
                else if (e == 'b') c = '\b';
                else if (e == 'f') c = '\f';
                else if (e == 'u') {
                    if (i + 4 > s.size()) return false;
                    const unsigned cp = (unsigned)std::stoul(s.substr(i, 4), nullptr, 16);
                    i += 4;
                    c = cp < 128 ? (char)cp : '?';   // names and paths here are ASCII
                } else c = e;
            }
            out.push_back(c);
        }
        if (i >= s.size()) return false;
        ++i;
        return true;
    }
    bool value(JVal& v, int depth = 0) {
        if (depth > 64) { err = "JSON nested too deeply"; return false; }
        ws();
        if (i >= s.size()) { err = "unexpected end of JSON"; return false; }
        const char c = s[i];
        if (c == '{') {
            ++i;
            v.kind = JVal::Obj;
            ws();
            if (i < s.size() && s[i] == '}') { ++i; return true; }
            for (;;) {
                ws();
                std::string key;
                if (!string(key)) { err = "expected a key"; return false; }
                ws();
                if (i >= s.size() || s[i] != ':') { err = "expected ':'"; return false; }
                ++i;
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.obj.emplace_back(std::move(key), std::move(child));
                ws();
                if (i < s.size() && s[i] == ',') { ++i; continue; }
                if (i < s.size() && s[i] == '}') { ++i; return true; }
                err = "expected ',' or '}'";
                return false;
            }
        }
        if (c == '[') {
            ++i;
            v.kind = JVal::Arr;
            ws();
            if (i < s.size() && s[i] == ']') { ++i; return true; }
            for (;;) {
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.arr.push_back(std::move(child));
                ws();
                if (i < s.size() && s[i] == ',') { ++i; continue; }
                if (i < s.size() && s[i] == ']') { ++i; return true; }
                err = "expected ',' or ']'";
                return false;
            }
        }
        if (c == '"') {
            v.kind = JVal::Str;
            if (!string(v.str)) { err = "bad string"; return false; }
            return true;
        }
        if (lit("true")) { v.kind = JVal::Bool; v.b = true; return true; }
        if (lit("false")) { v.kind = JVal::Bool; v.b = false; return true; }
        if (lit("null")) { v.kind = JVal::Null; return true; }
        size_t j = i;
        if (j < s.size() && (s[j] == '-' || s[j] == '+')) ++j;
        while (j < s.size() && (std::isdigit((unsigned char)s[j]) || s[j] == '.' || s[j] == 'e' || s[j] == 'E' ||
                                s[j] == '-' || s[j] == '+'))
            ++j;
        if (j == i) { err = "unexpected character in JSON"; return false; }
        v.kind = JVal::Num;
        v.num = std::strtod(s.substr(i, j - i).c_str(), nullptr);
        i = j;
        return true;
    }
};

// rescale / translate of load_scene.cpp:11-81, on float positions
void rescale(std::vector<float>& p, const JVal& box) {
    const JVal* mn = box.get("min");
    const JVal* mx = box.get("max");
    if (!mn || !mx) return;
    const double b0[3] = {mn->number("x", 0), mn->number("y", 0), mn->number("z", 0)};
    const double b1[3] = {mx->number("x", 0), mx->number("y", 0), mx->number("z", 0)};
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = std::numeric_limits<float>::max();
        hi[k] = std::numeric_limits<float>::lowest();
    }
    for (size_t i = 0; i < p.size(); i += 3)
        for (int k = 0; k < 3; ++k) {
            const float x = p[i + k];
            if (x < lo[k]) lo[k] = x;
            if (x > hi[k]) hi[k] = x;
        }
    for (size_t i = 0; i < p.size(); i += 3)
        for (int k = 0; k < 3; ++k) {
            const double d = hi[k] - lo[k];
            const float x0 = p[i + k];
            const double x = std::abs(d) < 1e-8 ? x0 : b0[k] + (b1[k] - b0[k]) * (x0 - lo[k]) / d;
            p[i + k] = (float)x;
        }
}

void translate(std::vector<float>& p, const JVal& t) {
    const float d[3] = {(float)t.number("x", 0), (float)t.number("y", 0), (float)t.number("z", 0)};
    for (size_t i = 0; i < p.size(); i += 3)
        for (int k = 0; k < 3; ++k) p[i + k] = p[i + k] + d[k];
}

std::string join_path(const std::string& json_path, const std::string& rel) {
    if (!rel.empty() && rel[0] == '/') return rel;
    const size_t slash = json_path.find_last_of('/');
    return slash == std::string::npos ? rel : json_path.substr(0, slash + 1) + rel;
}

bool is_ply(const std::string& p) { return p.size() > 4 && p.compare(p.size() - 4, 4, ".ply") == 0; }

}  // namespace

extern "C" sbs_status sbs_gpu_load_scene(sbs_gpu* h, const char* json_path, const sbs_gpu_material* material,
                                         const uint32_t env_cells[3], double env_margin, int32_t* first_body,
                                         int32_t* n_bodies) {
    if (!h || !json_path || !material || !env_cells || !(env_margin >= 0.0)) return SBS_EINVAL;
    std::ifstream f(json_path, std::ios::binary);
    if (!f) return SBS_EINVAL;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    JParser jp(text);
    JVal root;
    if (!jp.value(root) || root.kind != JVal::Obj) return SBS_EINVAL;
    int32_t first = -1, count = 0;
    // environment bodies (load_scene.cpp:170-233): collideable triangle meshes
    if (const JVal* env = root.get("environment"))
        for (const JVal& e : env->arr) {
            const JVal* geo = e.get("geometry");
            const JVal* path = geo ? geo->get("path") : nullptr;
            if (!path || path->kind != JVal::Str || !is_ply(path->str)) continue;
            PlyData d;
            std::string err;
            if (!read_ply(join_path(json_path, path->str), d, err)) continue;
            if (const JVal* box = e.get("box")) rescale(d.positions, *box);
            if (const JVal* tr = e.get("translation")) translate(d.positions, *tr);
            const JVal* col = e.get("collideable");
            if (!(col && col->kind == JVal::Bool && col->b) || d.tris.empty()) continue;
            std::vector<double> v(d.positions.begin(), d.positions.end());
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (size_t i = 0; i < v.size(); i += 3)
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], v[i + k]);
                    hi[k] = std::max(hi[k], v[i + k]);
                }
            for (int k = 0; k < 3; ++k) {
                lo[k] -= env_margin;
                hi[k] += env_margin;
            }
            const sbs_status s = sbs_gpu_add_environment_mesh(h, v.data(), (uint32_t)(v.size() / 3), d.tris.data(),
                                                              (uint32_t)(d.tris.size() / 3), lo, hi, env_cells);
            if (s) return s;
        }
    // soft objects (load_scene.cpp:235-361)
    if (const JVal* objs = root.get("objects"))
        for (const JVal& o : objs->arr) {
            const JVal* geo = o.get("geometry");
            const JVal* path = geo ? geo->get("path") : nullptr;
            if (!path || path->kind != JVal::Str || !is_ply(path->str)) continue;
            const JVal* phys = o.get("physics");
            PlyData d;
            std::string err;
            if (!read_ply(join_path(json_path, path->str), d, err)) continue;
            if (d.tets.empty()) continue;
            if (const JVal* box = o.get("box")) rescale(d.positions, *box);
            if (const JVal* tr = o.get("translation")) translate(d.positions, *tr);
            sbs_gpu_material m = *material;
            if (phys) m.density = phys->number("mass", m.density);
            std::vector<double> x0(d.positions.begin(), d.positions.end());
            int32_t body = -1;
            sbs_status s = sbs_gpu_add_body(h, x0.data(), nullptr, (uint32_t)(x0.size() / 3), d.tets.data(),
                                            (uint32_t)(d.tets.size() / 4), &m, nullptr, &body);
            if (s) return s;
            if (phys)
                if (const JVal* vel = phys->get("velocity")) {
                    const double v[3] = {vel->number("x", 0), vel->number("y", 0), vel->number("z", 0)};
                    if ((s = sbs_gpu_set_body_velocity(h, body, v)) != SBS_OK) return s;
                }
            if (first < 0) first = body;
            ++count;
        }
    if (first_body) *first_body = first;
    if (n_bodies) *n_bodies = count;
    return SBS_OK;
}
