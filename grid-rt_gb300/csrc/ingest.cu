// ingest.cu -- scene ingest: OBJ / PLY files to the triangle arrays the grid
// build takes, with the reference's Context semantics.
//
// The reference reads meshes through its rtdb loaders and builds geometry
// with rt::PrimitiveBuilder:
//   ObjFileLoader (src/rtdb/ObjFileLoader.cpp): each face's corners are
//     emitted as new vertices (Context::addVertex), a 3-corner face as
//     RT_TRIANGLES, a larger one as RT_POLYGON;
//   TriMeshLoader (src/rtdb/TriMeshLoader.cpp:17-84): PLY read into a
//     triangle mesh, three new vertices per triangle;
//   PrimitiveBuilder::updateTriangles / updatePolygonOrFan
//     (src/rtcore/PrimitiveBuilder.cpp): triangles (v0, v1, v2) / fans
//     (s, s+i, s+i+1);
//   PrimitiveBuilder::storeValidTriangle: a triangle whose Wald record
//     (TriAccel::buildFrom / valid, src/rtcore/Triangle.cpp:11-63) holds an
//     inf or NaN is dropped and the following ones renumbered -- its
//     vertices stay in the vertex array (they still count for the scene box).
// So ids of a loaded mesh are the reference's triangle ids.  The OBJ / PLY
// parsers themselves (objparser, trimesh2) are not in the reference checkout;
// these follow the published formats, PLY polygons split as fans.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "scene.h"

using namespace gridrt;

namespace {

rtg_status mfail(rtg_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

// The whole file in memory (NUL-terminated by std::string): the parsers
// below scan it in place instead of reading it a value at a time.
bool read_file(const char* path, std::string& buf) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    buf.clear();
    char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.append(chunk, n);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

inline bool is_space(char c) { return std::isspace((unsigned char)c) != 0; }

struct Builder {
    std::vector<float> verts;
    std::vector<int32_t> tris;
    std::vector<int64_t> face;
    int64_t dropped = 0;

    // TriAccel::buildFrom + valid: every record word finite.
    static bool valid(const float* v0, const float* v1, const float* v2) {
        const float b[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
        const float c[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
        const float n[3] = {c[1] * b[2] - c[2] * b[1], c[2] * b[0] - c[0] * b[2], c[0] * b[1] - c[1] * b[0]};
        int k;
        if (std::fabs(n[0]) > std::fabs(n[1]) && std::fabs(n[0]) > std::fabs(n[2])) k = 0;
        else if (std::fabs(n[1]) > std::fabs(n[2])) k = 1;
        else k = 2;
        const int u = (k + 1) % 3, v = (k + 2) % 3;
        const float inv_nk = 1.0f / n[k];
        const float nl[3] = {n[0] * inv_nk, n[1] * inv_nk, n[2] * inv_nk};
        float w[9];
        w[0] = n[u] / n[k];
        w[1] = n[v] / n[k];
        w[2] = v0[0] * nl[0] + v0[1] * nl[1] + v0[2] * nl[2];
        const float inv_den = 1.0f / (b[u] * c[v] - b[v] * c[u]);
        w[3] = -b[v] * inv_den;
        w[4] = b[u] * inv_den;
        w[5] = (b[v] * v0[u] - b[u] * v0[v]) * inv_den;
        w[6] = c[v] * inv_den;
        w[7] = -c[u] * inv_den;
        w[8] = (c[u] * v0[v] - c[v] * v0[u]) * inv_den;
        for (float x : w)
            if (!std::isfinite(x)) return false;
        return true;
    }

    int64_t add_vertex(const float* p) {
        verts.insert(verts.end(), p, p + 3);
        return (int64_t)verts.size() / 3 - 1;
    }

    void add_triangle(int64_t a, int64_t b, int64_t c, int64_t f) {
        if (!valid(&verts[3 * a], &verts[3 * b], &verts[3 * c])) {
            ++dropped;
            return;
        }
        tris.push_back((int32_t)a);
        tris.push_back((int32_t)b);
        tris.push_back((int32_t)c);
        face.push_back(f);
    }
};

// ---- OBJ -------------------------------------------------------------------
rtg_status load_obj(const char* path, Builder& B, int64_t* faces) {
    std::string buf;
    if (!read_file(path, buf)) return mfail(RTG_INVALID_PARAM, std::string("cannot open ") + path);
    std::vector<float> pos;
    int64_t f = 0, lineno = 0;
    std::vector<int64_t> corner;
    const char* p = buf.c_str();
    const char* const end = p + buf.size();
    B.verts.reserve(buf.size() / 8);
    while (p < end) {
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        const char* le = nl ? nl : end;   // the line is [p, le)
        ++lineno;
        const char* q = p;
        while (q < le && is_space(*q)) ++q;
        if (q + 1 < le && q[0] == 'v' && is_space(q[1])) {
            char* e = nullptr;
            const double x = std::strtod(q + 1, &e);
            const double y = std::strtod(e, &e);
            const double z = std::strtod(e, &e);
            pos.push_back((float)x);
            pos.push_back((float)y);
            pos.push_back((float)z);
        } else if (q + 1 < le && q[0] == 'f' && is_space(q[1])) {
            corner.clear();
            const int64_t nv = (int64_t)pos.size() / 3;
            const char* t = q + 1;
            for (;;) {
                while (t < le && is_space(*t)) ++t;
                if (t >= le) break;
                // one token: "v", "v/t", "v//n" or "v/t/n"; the vertex is its leading integer
                const long long r = std::strtoll(t, nullptr, 10);
                const long long idx = r > 0 ? r - 1 : nv + r;   // negative: relative to the end
                if (r == 0 || idx < 0 || idx >= nv)
                    return mfail(RTG_INVALID_GEOMETRY, "obj line " + std::to_string(lineno) + ": bad vertex index");
                corner.push_back(idx);
                while (t < le && !is_space(*t)) ++t;
            }
            if (corner.size() < 3)
                return mfail(RTG_INVALID_GEOMETRY, "obj line " + std::to_string(lineno) + ": face with < 3 corners");
            // Context::addVertex per corner, then the primitive's triangles
            const int64_t s0 = (int64_t)B.verts.size() / 3;
            for (int64_t c : corner) B.add_vertex(&pos[3 * c]);
            if (corner.size() == 3) {
                B.add_triangle(s0, s0 + 1, s0 + 2, f);
            } else {
                for (int64_t k = 1; k + 1 < (int64_t)corner.size(); ++k) B.add_triangle(s0, s0 + k, s0 + k + 1, f);
            }
            ++f;
        }
        p = nl ? nl + 1 : end;
    }
    *faces = f;
    return RTG_OK;
}

// ---- PLY -------------------------------------------------------------------
enum PlyType { P_NONE, P_I8, P_U8, P_I16, P_U16, P_I32, P_U32, P_F32, P_F64 };

PlyType ply_type(const std::string& t) {
    if (t == "char" || t == "int8") return P_I8;
    if (t == "uchar" || t == "uint8") return P_U8;
    if (t == "short" || t == "int16") return P_I16;
    if (t == "ushort" || t == "uint16") return P_U16;
    if (t == "int" || t == "int32") return P_I32;
    if (t == "uint" || t == "uint32") return P_U32;
    if (t == "float" || t == "float32") return P_F32;
    if (t == "double" || t == "float64") return P_F64;
    return P_NONE;
}

int ply_size(PlyType t) {
    switch (t) {
        case P_I8: case P_U8: return 1;
        case P_I16: case P_U16: return 2;
        case P_I32: case P_U32: case P_F32: return 4;
        case P_F64: return 8;
        default: return 0;
    }
}

struct PlyProp {
    std::string name;
    PlyType type = P_NONE;
    PlyType count = P_NONE;   // list count type, P_NONE for a scalar
};

struct PlyElem {
    std::string name;
    int64_t n = 0;
    std::vector<PlyProp> props;
};

struct PlyReader {
    const char* p;     // next byte of the body
    const char* end;
    int format;        // 0 ascii, 1 binary little endian, 2 binary big endian
    bool swap;         // binary byte order differs from the host's
    PlyReader(const char* begin, const char* e, int fmt) : p(begin), end(e), format(fmt) {
        const uint16_t one = 1;
        const bool host_le = *reinterpret_cast<const unsigned char*>(&one) == 1;
        swap = fmt != 0 && (fmt == 1) != host_le;
    }

    bool read(PlyType t, double* out) {
        if (format == 0) {
            char* e = nullptr;
            *out = std::strtod(p, &e);   // skips leading white space; the buffer is NUL-terminated
            if (e == p) return false;
            p = e;
            return true;
        }
        const int n = ply_size(t);
        if (n == 0 || end - p < n) return false;
        unsigned char b[8];
        std::memcpy(b, p, (size_t)n);
        p += n;
        if (swap)
            for (int i = 0; i < n / 2; ++i) std::swap(b[i], b[n - 1 - i]);
        switch (t) {
            case P_I8: *out = (double)(int8_t)b[0]; break;
            case P_U8: *out = (double)b[0]; break;
            case P_I16: { int16_t v; std::memcpy(&v, b, 2); *out = v; break; }
            case P_U16: { uint16_t v; std::memcpy(&v, b, 2); *out = v; break; }
            case P_I32: { int32_t v; std::memcpy(&v, b, 4); *out = v; break; }
            case P_U32: { uint32_t v; std::memcpy(&v, b, 4); *out = v; break; }
            case P_F32: { float v; std::memcpy(&v, b, 4); *out = v; break; }
            case P_F64: { double v; std::memcpy(&v, b, 8); *out = v; break; }
            default: return false;
        }
        return true;
    }
};

rtg_status load_ply(const char* path, Builder& B, int64_t* faces) {
    std::string buf;
    if (!read_file(path, buf)) return mfail(RTG_INVALID_PARAM, std::string("cannot open ") + path);
    // header lines up to end_header; the body starts after its newline
    const char* cur = buf.c_str();
    const char* const bend = cur + buf.size();
    auto next_line = [&](std::string& line) -> bool {
        if (cur >= bend) return false;
        const char* nl = static_cast<const char*>(std::memchr(cur, '\n', (size_t)(bend - cur)));
        const char* le = nl ? nl : bend;
        line.assign(cur, le);
        cur = nl ? nl + 1 : bend;
        return true;
    };
    std::string line;
    if (!next_line(line) || line.compare(0, 3, "ply") != 0) return mfail(RTG_INVALID_GEOMETRY, "not a PLY file");
    int format = -1;
    std::vector<PlyElem> elems;
    while (next_line(line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ss(line);
        std::string kw;
        ss >> kw;
        if (kw == "format") {
            std::string f;
            ss >> f;
            format = f == "ascii" ? 0 : (f == "binary_little_endian" ? 1 : (f == "binary_big_endian" ? 2 : -1));
        } else if (kw == "element") {
            PlyElem e;
            ss >> e.name >> e.n;
            elems.push_back(e);
        } else if (kw == "property") {
            if (elems.empty()) return mfail(RTG_INVALID_GEOMETRY, "ply: property before element");
            PlyProp p;
            std::string t;
            ss >> t;
            if (t == "list") {
                std::string ct, it;
                ss >> ct >> it >> p.name;
                p.count = ply_type(ct);
                p.type = ply_type(it);
                if (p.count == P_NONE || p.type == P_NONE) return mfail(RTG_INVALID_GEOMETRY, "ply: bad list type");
            } else {
                p.type = ply_type(t);
                ss >> p.name;
                if (p.type == P_NONE) return mfail(RTG_INVALID_GEOMETRY, "ply: bad property type");
            }
            elems.back().props.push_back(p);
        } else if (kw == "end_header") {
            break;
        }
    }
    if (format < 0) return mfail(RTG_INVALID_GEOMETRY, "ply: missing or unknown format");
    PlyReader R(cur, bend, format);
    std::vector<float> pos;
    for (const PlyElem& e : elems) {
        // room for every vertex and, for triangles, their three new vertices each
        if (e.name == "vertex" && e.n > 0 && e.n < (int64_t(1) << 31)) pos.reserve(3 * (size_t)e.n);
        if (e.name == "face" && e.n > 0 && e.n < (int64_t(1) << 31)) {
            B.verts.reserve(9 * (size_t)e.n);
            B.tris.reserve(3 * (size_t)e.n);
            B.face.reserve((size_t)e.n);
        }
    }
    std::vector<int64_t> poly;
    int64_t f = 0;
    for (const PlyElem& e : elems) {
        int ix = -1, iy = -1, iz = -1, ifc = -1;
        for (size_t k = 0; k < e.props.size(); ++k) {
            const std::string& nm = e.props[k].name;
            if (nm == "x") ix = (int)k;
            if (nm == "y") iy = (int)k;
            if (nm == "z") iz = (int)k;
            if ((nm == "vertex_indices" || nm == "vertex_index") && e.props[k].count != P_NONE) ifc = (int)k;
        }
        const bool is_vertex = e.name == "vertex";
        const bool is_face = e.name == "face";
        if (is_vertex && (ix < 0 || iy < 0 || iz < 0)) return mfail(RTG_INVALID_GEOMETRY, "ply: vertex without x y z");
        if (is_face && ifc < 0) return mfail(RTG_INVALID_GEOMETRY, "ply: face without vertex_indices");
        for (int64_t r = 0; r < e.n; ++r) {
            float p[3] = {0.f, 0.f, 0.f};
            for (size_t k = 0; k < e.props.size(); ++k) {
                const PlyProp& pr = e.props[k];
                if (pr.count != P_NONE) {
                    double cnt = 0;
                    if (!R.read(pr.count, &cnt) || cnt < 0) return mfail(RTG_INVALID_GEOMETRY, "ply: truncated list");
                    if ((int)k == ifc) poly.clear();
                    for (int64_t q = 0; q < (int64_t)cnt; ++q) {
                        double v = 0;
                        if (!R.read(pr.type, &v)) return mfail(RTG_INVALID_GEOMETRY, "ply: truncated list");
                        if ((int)k == ifc) poly.push_back((int64_t)v);
                    }
                } else {
                    double v = 0;
                    if (!R.read(pr.type, &v)) return mfail(RTG_INVALID_GEOMETRY, "ply: truncated data");
                    if ((int)k == ix) p[0] = (float)v;
                    if ((int)k == iy) p[1] = (float)v;
                    if ((int)k == iz) p[2] = (float)v;
                }
            }
            if (is_vertex) pos.insert(pos.end(), p, p + 3);
            if (is_face) {
                const int64_t nv = (int64_t)pos.size() / 3;
                if (poly.size() < 3) return mfail(RTG_INVALID_GEOMETRY, "ply: face with < 3 vertices");
                for (int64_t q : poly)
                    if (q < 0 || q >= nv) return mfail(RTG_INVALID_GEOMETRY, "ply: bad vertex index");
                // triangles (fan), three new vertices each
                for (size_t k = 1; k + 1 < poly.size(); ++k) {
                    const int64_t a = B.add_vertex(&pos[3 * poly[0]]);
                    const int64_t b = B.add_vertex(&pos[3 * poly[k]]);
                    const int64_t c = B.add_vertex(&pos[3 * poly[k + 1]]);
                    B.add_triangle(a, b, c, f);
                }
                ++f;
            }
        }
    }
    *faces = f;
    return RTG_OK;
}

bool ends_with(const std::string& s, const char* suf) {
    const size_t n = std::strlen(suf);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)s[s.size() - n + i]) != suf[i]) return false;
    return true;
}

}  // namespace

extern "C" {

rtg_status rtg_mesh_load(const char* path, rtg_mesh* out) {
    if (!path || !out) return mfail(RTG_INVALID_PARAM, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    Builder B;
    int64_t faces = 0;
    const std::string p(path);
    rtg_status rc;
    if (ends_with(p, ".obj")) rc = load_obj(path, B, &faces);
    else if (ends_with(p, ".ply")) rc = load_ply(path, B, &faces);
    else return mfail(RTG_INVALID_PARAM, "mesh file must end in .obj or .ply");
    if (rc) return rc;
    if ((int64_t)B.verts.size() / 3 > 0x7fffffffLL) return mfail(RTG_INVALID_GEOMETRY, "mesh exceeds int32 indices");
    out->nverts = (int64_t)B.verts.size() / 3;
    out->ntris = (int64_t)B.tris.size() / 3;
    out->faces = faces;
    out->dropped = B.dropped;
    out->verts = static_cast<float*>(std::malloc(sizeof(float) * (B.verts.size() + 1)));
    out->tris = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * (B.tris.size() + 1)));
    out->source_face = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (B.face.size() + 1)));
    if (!out->verts || !out->tris || !out->source_face) {
        rtg_mesh_free(out);
        return mfail(RTG_NO_MEMORY, "mesh arrays");
    }
    std::memcpy(out->verts, B.verts.data(), sizeof(float) * B.verts.size());
    std::memcpy(out->tris, B.tris.data(), sizeof(int32_t) * B.tris.size());
    std::memcpy(out->source_face, B.face.data(), sizeof(int64_t) * B.face.size());
    return RTG_OK;
}

void rtg_mesh_free(rtg_mesh* m) {
    if (!m) return;
    std::free(m->verts);
    std::free(m->tris);
    std::free(m->source_face);
    std::memset(m, 0, sizeof(*m));
}

rtg_status rtg_scene_load(rtg_scene scene, const char* path, rtg_mesh* info) {
    if (!scene) return mfail(RTG_INVALID_PARAM, "scene is NULL");
    rtg_mesh m;
    rtg_status rc = rtg_mesh_load(path, &m);
    if (rc) return rc;
    rc = rtg_scene_set_geometry(scene, m.verts, m.nverts, m.tris, m.ntris, nullptr);
    if (info) {
        *info = m;
        std::free(m.verts);
        std::free(m.tris);
        info->verts = nullptr;
        info->tris = nullptr;   // source_face stays with the caller (rtg_mesh_free)
    } else {
        rtg_mesh_free(&m);
    }
    return rc;
}

}  // extern "C"
