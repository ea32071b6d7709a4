// gbr_obj.cpp -- Wavefront OBJ reader with tangent generation, restating the
// reference's ObjParser (ObjParser.cpp) for meshes that feed gbr_mesh_upload.
//
// The reference's line grammar is kept as it is, quirks included, so a file
// reads into the same vertices, indices and vertex type:
//   * a line is split at '\n' ('\r' stays); empty lines and lines starting
//     with '#' are skipped; the prefix is the text before the first ' '
//     (ObjParser.cpp:34-41);
//   * "v", "vt", "vn" drop their first 3 characters and "f" its first 2
//     (:42-62): "v  x y z" (3ds Max's two spaces) reads as written, while
//     "v x y z" loses the first character of x -- as in the reference;
//   * fields are separated by single spaces (std::getline on ' ', :196-205)
//     and converted like std::stof / std::stoi (leading blanks skipped, the
//     longest number prefix taken); a field with no number is an error here
//     (std::stof throws in the reference);
//   * a face reads its first three space-separated fields; each splits at
//     '/' (:135-148) and its indices (1-based) go round-robin to position,
//     uv and normal lists by their order within the face (:166-181);
//   * "vt" keeps u and v, v -> 1 - v when the y axis is inverted (:188-194);
//     "vn" is normalised (:183-187).
// Vertices are then built as AssignVertices (pointer form, :216-355) does:
// each face corner becomes a vertex unless an earlier one has the same
// position index, the same uv index and an equal normal (AreEqual, 2 ulp,
// MathUtilities.h:29-38) -- the first such earlier vertex is reused; with
// uvs and normals, per-triangle tangents are summed into the vertices and
// each sum is normalised after rejecting its normal component (:280-305).
// Where the reference reads memory it never set, this reader sets a value
// and says so: tangents start at 0 and colours at (1, 1, 1) (IVertex() is
// "purposely uninitialized", Vertex.h:115-117); with uvs but no normals the
// normal is 0 (the reference indexes an empty normal list, :330); normals
// without uvs are kept, matched like positions + normals (the reference
// fills no vertex at all for that case); the vertex count is the number of
// distinct vertices (the reference reports the face count outside the
// uv + normal case, :218, :316).
// All float arithmetic is single precision, one rounding per operation in
// the reference's order (the library is built with -ffp-contract=off).
#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gbr.h"

namespace gbr {
void set_last_error(const char* msg);   // gbr_last_error_string()
}

namespace {

struct V3 {
    float x, y, z;
};

bool are_equal(float a, float b) {   // AreEqual<float>(a, b, 2)
    const float d = std::fabs(a - b);
    return d <= FLT_EPSILON * std::fabs(a + b) * 2.f || d < FLT_MIN;
}

V3 normalized(V3 v) {   // GetNormalized (Vector.h:41-64)
    const float m = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    if (m == 0.f) return V3{0.f, 0.f, 0.f};
    const float inv = 1.f / m;
    return V3{v.x * inv, v.y * inv, v.z * inv};
}

struct Parsed {
    std::vector<V3> positions, normals;
    std::vector<float> uvs;   // u, v pairs
    std::vector<unsigned> pos_idx, uv_idx, norm_idx;
    unsigned faces = 0;
};

// The fields of `s` separated by single spaces, as std::getline(ss, f, ' ')
// returns them: at most `max` fields, an absent field is empty.
void fields(const std::string& s, std::string* out, int max) {
    size_t at = 0;
    for (int k = 0; k < max; ++k) {
        if (at > s.size()) { out[k].clear(); continue; }
        const size_t sp = s.find(' ', at);
        if (sp == std::string::npos) {
            out[k] = s.substr(at);
            at = s.size() + 1;
        } else {
            out[k] = s.substr(at, sp - at);
            at = sp + 1;
        }
    }
}

bool to_float(const std::string& f, float& v) {   // std::stof
    const char* b = f.c_str();
    char* e = nullptr;
    errno = 0;
    v = std::strtof(b, &e);
    return e != b && errno != ERANGE;
}

bool to_int(const std::string& f, long& v) {   // std::stoi
    const char* b = f.c_str();
    char* e = nullptr;
    errno = 0;
    v = std::strtol(b, &e, 10);
    return e != b && errno != ERANGE && v >= -2147483648L && v <= 2147483647L;
}

gbr_status fail_at(size_t line, const char* what) {
    char msg[160];
    if (line) std::snprintf(msg, sizeof msg, "OBJ line %zu: %s", line, what);
    else std::snprintf(msg, sizeof msg, "OBJ: %s", what);
    gbr::set_last_error(msg);
    return GBR_ERR_INVALID_ARG;
}

gbr_status parse(const char* text, size_t length, bool invert_y, Parsed& P) {
    size_t line_no = 0, at = 0;
    std::string line;
    while (at < length) {   // std::getline on '\n'
        const char* nl = static_cast<const char*>(std::memchr(text + at, '\n', length - at));
        const size_t end = nl ? (size_t)(nl - text) : length;
        line.assign(text + at, end - at);
        at = end + 1;
        ++line_no;
        if (line.empty() || line[0] == '#') continue;
        const size_t sp = line.find(' ');
        const std::string prefix = sp == std::string::npos ? line : line.substr(0, sp);
        std::string f[3];
        if (prefix == "v" || prefix == "vt" || prefix == "vn") {
            if (line.size() < 3) return fail_at(line_no, "field missing");
            fields(line.substr(3), f, 3);
            if (prefix == "vt") {
                float u, v;
                if (!to_float(f[1], v) || !to_float(f[0], u)) return fail_at(line_no, "uv field is not a number");
                if (invert_y) v = 1.f - v;
                P.uvs.push_back(u);
                P.uvs.push_back(v);
                continue;
            }
            V3 p;
            if (!to_float(f[0], p.x) || !to_float(f[1], p.y) || !to_float(f[2], p.z))
                return fail_at(line_no, "coordinate is not a number");
            if (prefix == "v") P.positions.push_back(p);
            else P.normals.push_back(normalized(p));
        } else if (prefix == "f") {
            if (line.size() < 2) return fail_at(line_no, "field missing");
            fields(line.substr(2), f, 3);
            std::vector<long> idx;
            for (int i = 0; i < 3; ++i) {
                // ObjParser.cpp:135-148: the corner's indices, split at '/'
                const std::string& c = f[i];
                size_t start = 0, slash = 0;
                for (;;) {
                    const size_t cut = c.find('/', start);
                    long v;
                    if (!to_int(c.substr(start, cut == std::string::npos ? std::string::npos : cut - start), v))
                        return fail_at(line_no, "face index is not a number");
                    idx.push_back(v - 1);
                    slash = c.find('/', slash + 1);
                    if (slash == std::string::npos) break;
                    start = slash + 1;
                }
            }
            const size_t per = idx.size() / 3;
            for (size_t k = 0; k < idx.size(); ++k) {
                if (idx[k] < 0) return fail_at(line_no, "face index below 1");
                switch (k % per) {
                    case 0: P.pos_idx.push_back((unsigned)idx[k]); break;
                    case 1: P.uv_idx.push_back((unsigned)idx[k]); break;
                    case 2: P.norm_idx.push_back((unsigned)idx[k]); break;
                    default: break;
                }
            }
            ++P.faces;
        }
        // "o", "g" and unknown prefixes are reported by the reference and skipped
    }
    return GBR_OK;
}

gbr_status assemble(const Parsed& P, gbr_obj_mesh* out) {
    const size_t n = P.pos_idx.size();
    const bool uvs = !P.uvs.empty(), norms = !P.normals.empty();
    if (uvs && P.uv_idx.size() < n) return fail_at(0, "a face lacks uv indices");
    if (norms && P.norm_idx.size() < n) return fail_at(0, "a face lacks normal indices");
    for (size_t i = 0; i < n; ++i) {
        if (P.pos_idx[i] >= P.positions.size()) return fail_at(0, "position index out of range");
        if (uvs && 2u * (size_t)P.uv_idx[i] >= P.uvs.size()) return fail_at(0, "uv index out of range");
        if (norms && P.norm_idx[i] >= P.normals.size()) return fail_at(0, "normal index out of range");
    }
    std::vector<gbr_ivertex> verts;
    std::vector<uint32_t> index(n);
    // earlier vertices by (position, uv) index, in creation order
    std::unordered_map<unsigned long long, std::vector<uint32_t>> seen;
    for (size_t i = 0; i < n; ++i) {
        const unsigned pi = P.pos_idx[i], ti = uvs ? P.uv_idx[i] : 0u;
        const unsigned long long key = ((unsigned long long)pi << 32) | ti;
        std::vector<uint32_t>& cand = seen[key];
        const V3* nrm = norms ? &P.normals[P.norm_idx[i]] : nullptr;
        uint32_t found = 0xFFFFFFFFu;
        for (uint32_t c : cand) {
            if (nrm) {
                const gbr_ivertex& o = verts[c];
                if (!(are_equal(o.n[0], nrm->x) && are_equal(o.n[1], nrm->y) && are_equal(o.n[2], nrm->z))) continue;
            }
            found = c;
            break;
        }
        if (found == 0xFFFFFFFFu) {
            gbr_ivertex v;
            std::memset(&v, 0, sizeof v);
            const V3& p = P.positions[pi];
            v.p[0] = p.x; v.p[1] = p.y; v.p[2] = p.z;
            if (uvs) { v.uv[0] = P.uvs[2u * ti]; v.uv[1] = P.uvs[2u * ti + 1u]; }
            if (nrm) { v.n[0] = nrm->x; v.n[1] = nrm->y; v.n[2] = nrm->z; }
            v.c[0] = v.c[1] = v.c[2] = 1.f;
            found = (uint32_t)verts.size();
            verts.push_back(v);
            cand.push_back(found);
        }
        index[i] = found;
    }
    int32_t type = 0;
    if (uvs) type |= GBR_VT_UV;
    if (norms) type |= GBR_VT_NORM;
    if (uvs && norms) {
        type |= GBR_VT_TAN;
        for (size_t i = 0; i + 2 < n; i += 3) {   // ObjParser.cpp:280-300
            gbr_ivertex& a = verts[index[i]];
            gbr_ivertex& b = verts[index[i + 1]];
            gbr_ivertex& c = verts[index[i + 2]];
            const V3 e0{b.p[0] - a.p[0], b.p[1] - a.p[1], b.p[2] - a.p[2]};
            const V3 e1{c.p[0] - a.p[0], c.p[1] - a.p[1], c.p[2] - a.p[2]};
            const float dx0 = b.uv[0] - a.uv[0], dx1 = c.uv[0] - a.uv[0];
            const float dy0 = b.uv[1] - a.uv[1], dy1 = c.uv[1] - a.uv[1];
            const float r = 1.f / (dx0 * dy1 - dx1 * dy0);
            const V3 t{(e0.x * dy1 - e1.x * dy0) * r, (e0.y * dy1 - e1.y * dy0) * r, (e0.z * dy1 - e1.z * dy0) * r};
            for (gbr_ivertex* v : {&a, &b, &c}) {
                v->tan[0] += t.x;
                v->tan[1] += t.y;
                v->tan[2] += t.z;
            }
        }
        for (gbr_ivertex& v : verts) {   // GetNormalized(Reject(tan, n)), Vector.h:66-74
            const V3 t{v.tan[0], v.tan[1], v.tan[2]}, nn{v.n[0], v.n[1], v.n[2]};
            const float s = (t.x * nn.x + t.y * nn.y + t.z * nn.z) / (nn.x * nn.x + nn.y * nn.y + nn.z * nn.z);
            const V3 rej{t.x - nn.x * s, t.y - nn.y * s, t.z - nn.z * s};
            const V3 u = normalized(rej);
            v.tan[0] = u.x; v.tan[1] = u.y; v.tan[2] = u.z;
        }
    }
    out->num_vertices = (uint32_t)verts.size();
    out->num_indices = (uint32_t)n;
    out->num_faces = P.faces;
    out->vertex_type = type;
    out->vertices = static_cast<gbr_ivertex*>(std::malloc(std::max<size_t>(verts.size(), 1) * sizeof(gbr_ivertex)));
    out->indices = static_cast<uint32_t*>(std::malloc(std::max<size_t>(n, 1) * sizeof(uint32_t)));
    if (!out->vertices || !out->indices) {
        std::free(out->vertices);
        std::free(out->indices);
        out->vertices = nullptr;
        out->indices = nullptr;
        return GBR_ERR_OUT_OF_MEMORY;
    }
    if (!verts.empty()) std::memcpy(out->vertices, verts.data(), verts.size() * sizeof(gbr_ivertex));
    if (n) std::memcpy(out->indices, index.data(), n * sizeof(uint32_t));
    return GBR_OK;
}

}  // namespace

extern "C" {

gbr_status gbr_obj_read_text(const char* text, size_t length, int invert_y, gbr_obj_mesh* out) {
    if (!out || (!text && length)) return fail_at(0, "null argument");
    std::memset(out, 0, sizeof *out);
    Parsed P;
    gbr_status st = parse(text, length, invert_y != 0, P);
    if (st != GBR_OK) return st;
    return assemble(P, out);
}

gbr_status gbr_obj_read_file(const char* path, int invert_y, gbr_obj_mesh* out) {
    if (!out || !path) return fail_at(0, "null argument");
    std::memset(out, 0, sizeof *out);
    // ObjParser::OpenFile (ObjParser.cpp:563-582): the text from the first
    // '.' on must be ".obj"
    const char* dot = std::strchr(path, '.');
    if (!dot || std::strcmp(dot, ".obj") != 0) return fail_at(0, "only '.obj' files are read");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) {
        gbr::set_last_error("cannot open the OBJ file");
        return GBR_ERR_NOT_FOUND;
    }
    std::string text;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, got);
    std::fclose(fp);
    return gbr_obj_read_text(text.data(), text.size(), invert_y, out);
}

void gbr_obj_free(gbr_obj_mesh* m) {
    if (!m) return;
    std::free(m->vertices);
    std::free(m->indices);
    std::memset(m, 0, sizeof *m);
}

}  // extern "C"
