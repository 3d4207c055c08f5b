// OBJ and glTF 2.0 loaders (see loaders.h).  Written from the file-format specifications (Wavefront OBJ;
// Khronos glTF 2.0 with KHR_materials_emissive_strength, KHR_materials_ior, KHR_materials_transmission)
// and the reference's use of their contents (src/scene/Models.cpp:117-175,
// src/scene/gltf/gltfloader.cpp:120-255, 380-430).
#include "loaders.h"

#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <tuple>
#include <unordered_map>

#include "errors.h"
#include "image.h"
#include "json.h"

namespace rt {

namespace {

std::vector<uint8_t> read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(REINA_ERR_IO, "cannot open " + path);
    std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    return data;
}

std::string dir_of(const std::string& path) {
    const size_t s = path.find_last_of('/');
    return s == std::string::npos ? std::string(".") : path.substr(0, s);
}

void norm3(float v[3]) {
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0.0f) { v[0] /= l; v[1] /= l; v[2] /= l; }
}

void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace

void tangent_frames(const std::vector<float>& pos4, const std::vector<float>& n3, const std::vector<float>& uv2,
                    const std::vector<uint32_t>& idx, std::vector<float>& tbn9) {
    const size_t nv = pos4.size() / 4;
    std::vector<double> tan(3 * nv, 0.0), bit(3 * nv, 0.0);
    const bool have_uv = uv2.size() >= 2 * nv;
    if (have_uv) {
        for (size_t t = 0; t + 2 < idx.size(); t += 3) {
            const uint32_t i0 = idx[t], i1 = idx[t + 1], i2 = idx[t + 2];
            if (i0 >= nv || i1 >= nv || i2 >= nv) continue;
            const double e1[3] = {pos4[4 * i1] - (double)pos4[4 * i0], pos4[4 * i1 + 1] - (double)pos4[4 * i0 + 1],
                                  pos4[4 * i1 + 2] - (double)pos4[4 * i0 + 2]};
            const double e2[3] = {pos4[4 * i2] - (double)pos4[4 * i0], pos4[4 * i2 + 1] - (double)pos4[4 * i0 + 1],
                                  pos4[4 * i2 + 2] - (double)pos4[4 * i0 + 2]};
            const double du1 = uv2[2 * i1] - (double)uv2[2 * i0], dv1 = uv2[2 * i1 + 1] - (double)uv2[2 * i0 + 1];
            const double du2 = uv2[2 * i2] - (double)uv2[2 * i0], dv2 = uv2[2 * i2 + 1] - (double)uv2[2 * i0 + 1];
            const double det = du1 * dv2 - du2 * dv1;
            if (std::fabs(det) < 1e-20) continue;
            const double r = 1.0 / det;
            double T[3], B[3];
            for (int k = 0; k < 3; ++k) {
                T[k] = (e1[k] * dv2 - e2[k] * dv1) * r;
                B[k] = (e2[k] * du1 - e1[k] * du2) * r;
            }
            for (uint32_t v : {i0, i1, i2})
                for (int k = 0; k < 3; ++k) {
                    tan[3 * v + k] += T[k];
                    bit[3 * v + k] += B[k];
                }
        }
    }
    tbn9.assign(9 * nv, 0.0f);
    for (size_t v = 0; v < nv; ++v) {
        float N[3] = {n3[3 * v], n3[3 * v + 1], n3[3 * v + 2]};
        float T[3] = {(float)tan[3 * v], (float)tan[3 * v + 1], (float)tan[3 * v + 2]};
        const float d = T[0] * N[0] + T[1] * N[1] + T[2] * N[2];
        for (int k = 0; k < 3; ++k) T[k] -= d * N[k];
        float l = std::sqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2]);
        if (!(l > 1e-12f)) {   // no UV gradient: any unit vector orthogonal to N
            const float a[3] = {std::fabs(N[0]) < 0.9f ? 1.0f : 0.0f, std::fabs(N[0]) < 0.9f ? 0.0f : 1.0f, 0.0f};
            cross3(a, N, T);
            l = std::sqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2]);
        }
        if (l > 0.0f)
            for (int k = 0; k < 3; ++k) T[k] /= l;
        float B[3];
        cross3(N, T, B);
        const double hand = B[0] * bit[3 * v] + B[1] * bit[3 * v + 1] + B[2] * bit[3 * v + 2];
        if (hand < 0.0)
            for (int k = 0; k < 3; ++k) B[k] = -B[k];
        for (int k = 0; k < 3; ++k) {
            tbn9[9 * v + k] = T[k];
            tbn9[9 * v + 3 + k] = B[k];
            tbn9[9 * v + 6 + k] = N[k];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// OBJ

ModelData parse_obj(const std::string& text, const std::string& name) {
    std::vector<float> P, T, N;   // file arrays (xyz, uv, xyz)
    struct Corner { int64_t v, t, n; };
    std::vector<Corner> corners;  // triangle corners, already fanned
    std::istringstream in(text);
    std::string line;
    size_t lineno = 0;
    auto resolve = [&](int64_t i, size_t count) -> int64_t {
        if (i > 0) return i - 1;
        if (i < 0) return (int64_t)count + i;
        return -1;
    };
    while (std::getline(in, line)) {
        ++lineno;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag)) continue;
        if (tag == "v") {
            float x, y, z;
            if (!(ls >> x >> y >> z)) fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": malformed vertex");
            P.insert(P.end(), {x, y, z});
        } else if (tag == "vt") {
            float u, v = 0.0f;
            if (!(ls >> u)) fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": malformed texture coordinate");
            ls >> v;
            T.insert(T.end(), {u, v});
        } else if (tag == "vn") {
            float x, y, z;
            if (!(ls >> x >> y >> z)) fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": malformed normal");
            N.insert(N.end(), {x, y, z});
        } else if (tag == "f") {
            std::vector<Corner> poly;
            std::string tok;
            while (ls >> tok) {
                Corner c{-1, -1, -1};
                int64_t vals[3] = {0, 0, 0};
                bool present[3] = {false, false, false};
                size_t part = 0, start = 0;
                for (size_t i = 0; i <= tok.size(); ++i) {
                    if (i == tok.size() || tok[i] == '/') {
                        if (part > 2) fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": malformed face");
                        if (i > start) {
                            vals[part] = std::stoll(tok.substr(start, i - start));
                            present[part] = true;
                        }
                        ++part;
                        start = i + 1;
                    }
                }
                if (!present[0]) fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": face corner without vertex");
                c.v = resolve(vals[0], P.size() / 3);
                c.t = present[1] ? resolve(vals[1], T.size() / 2) : -1;
                c.n = present[2] ? resolve(vals[2], N.size() / 3) : -1;
                if (c.v < 0 || (size_t)c.v >= P.size() / 3 || (present[1] && (c.t < 0 || (size_t)c.t >= T.size() / 2)) ||
                    (present[2] && (c.n < 0 || (size_t)c.n >= N.size() / 3)))
                    fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": face index out of range");
                poly.push_back(c);
            }
            if (poly.size() < 3) fail(REINA_ERR_IO, name + ":" + std::to_string(lineno) + ": face with fewer than 3 corners");
            for (size_t k = 1; k + 1 < poly.size(); ++k) {
                corners.push_back(poly[0]);
                corners.push_back(poly[k]);
                corners.push_back(poly[k + 1]);
            }
        }
        // o, g, s, usemtl, mtllib, l, p: not needed for geometry (all faces form one model)
    }
    if (corners.empty()) fail(REINA_ERR_IO, "no faces in " + name);
    bool has_uv = true, has_n = true;
    for (const Corner& c : corners) {
        has_uv = has_uv && c.t >= 0;
        has_n = has_n && c.n >= 0;
    }
    // one vertex per distinct (v, t, n) triple
    std::map<std::tuple<int64_t, int64_t, int64_t>, uint32_t> ids;
    ModelData m;
    std::vector<float> normals, uvs;
    std::vector<int64_t> src_pos;
    for (const Corner& c : corners) {
        const auto key = std::make_tuple(c.v, has_uv ? c.t : -1, has_n ? c.n : -1);
        auto it = ids.find(key);
        uint32_t id;
        if (it == ids.end()) {
            id = (uint32_t)src_pos.size();
            ids.emplace(key, id);
            src_pos.push_back(c.v);
            m.vertices.insert(m.vertices.end(), {P[3 * c.v], P[3 * c.v + 1], P[3 * c.v + 2], 1.0f});
            if (has_uv) uvs.insert(uvs.end(), {T[2 * c.t], 1.0f - T[2 * c.t + 1]});
            if (has_n) {
                float nn[3] = {N[3 * c.n], N[3 * c.n + 1], N[3 * c.n + 2]};
                normals.insert(normals.end(), nn, nn + 3);
            }
        } else {
            id = it->second;
        }
        m.indices.push_back(id);
    }
    const size_t nv = src_pos.size();
    if (!has_n) {   // smooth normals over all faces sharing a file position
        std::vector<double> acc(3 * (P.size() / 3), 0.0);
        for (size_t t = 0; t < m.indices.size(); t += 3) {
            const float* a = &m.vertices[4 * m.indices[t]];
            const float* b = &m.vertices[4 * m.indices[t + 1]];
            const float* c = &m.vertices[4 * m.indices[t + 2]];
            const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            float fn[3];
            cross3(e1, e2, fn);
            norm3(fn);
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) acc[3 * src_pos[m.indices[t + j]] + k] += fn[k];
        }
        normals.resize(3 * nv);
        for (size_t v = 0; v < nv; ++v) {
            float nn[3] = {(float)acc[3 * src_pos[v]], (float)acc[3 * src_pos[v] + 1], (float)acc[3 * src_pos[v] + 2]};
            norm3(nn);
            for (int k = 0; k < 3; ++k) normals[3 * v + k] = nn[k];
        }
    }
    if (has_uv) {
        tangent_frames(m.vertices, normals, uvs, m.indices, m.tbns);
        m.tex_coords = uvs;
        m.tex_indices = m.indices;
    } else {   // no UVs: the tangent and bitangent are zero, as the reference leaves them
        m.tbns.assign(9 * nv, 0.0f);
        for (size_t v = 0; v < nv; ++v)
            for (int k = 0; k < 3; ++k) m.tbns[9 * v + 6 + k] = normals[3 * v + k];
    }
    m.tbn_indices = m.indices;
    return m;
}

ModelData load_obj(const std::string& path) {
    const std::vector<uint8_t> d = read_file(path);
    return parse_obj(std::string(d.begin(), d.end()), path);
}

// ------------------------------------------------------------------------------------------------
// glTF 2.0

namespace {

std::vector<uint8_t> base64_decode(const std::string& s, size_t from) {
    static const std::vector<int8_t> table = [] {
        std::vector<int8_t> t(256, -1);
        const char* a = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
        for (int i = 0; i < 64; ++i) t[(uint8_t)a[i]] = (int8_t)i;
        return t;
    }();
    std::vector<uint8_t> out;
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = from; i < s.size(); ++i) {
        const char c = s[i];
        if (c == '=') break;
        const int v = table[(uint8_t)c];
        if (v < 0) {
            if (c == '\n' || c == '\r' || c == ' ') continue;
            fail(REINA_ERR_IO, "glTF: bad base64 data URI");
        }
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)((acc >> bits) & 0xFF));
        }
    }
    return out;
}

struct Gltf {
    Json doc;
    std::vector<std::vector<uint8_t>> buffers;
};

struct Accessor {
    const uint8_t* base = nullptr;
    size_t count = 0, stride = 0;
    int comps = 0, ctype = 0;
    bool normalized = false;

    float get(size_t i, int c) const {
        const uint8_t* p = base + i * stride;
        switch (ctype) {
            case 5126: { float f; std::memcpy(&f, p + 4 * c, 4); return f; }
            case 5121: { const float v = p[c]; return normalized ? v / 255.0f : v; }
            case 5120: { const float v = (int8_t)p[c]; return normalized ? std::fmax(v / 127.0f, -1.0f) : v; }
            case 5123: { uint16_t u; std::memcpy(&u, p + 2 * c, 2); return normalized ? u / 65535.0f : (float)u; }
            case 5122: { int16_t u; std::memcpy(&u, p + 2 * c, 2); return normalized ? std::fmax(u / 32767.0f, -1.0f) : (float)u; }
            case 5125: { uint32_t u; std::memcpy(&u, p + 4 * c, 4); return (float)u; }
        }
        return 0.0f;
    }
    uint32_t index(size_t i) const {
        const uint8_t* p = base + i * stride;
        if (ctype == 5121) return p[0];
        if (ctype == 5123) { uint16_t u; std::memcpy(&u, p, 2); return u; }
        uint32_t u; std::memcpy(&u, p, 4); return u;
    }
};

int type_comps(const std::string& t) {
    if (t == "SCALAR") return 1;
    if (t == "VEC2") return 2;
    if (t == "VEC3") return 3;
    if (t == "VEC4") return 4;
    if (t == "MAT4") return 16;
    return 0;
}

int ctype_size(int c) {
    switch (c) {
        case 5120: case 5121: return 1;
        case 5122: case 5123: return 2;
        case 5125: case 5126: return 4;
    }
    return 0;
}

Accessor accessor(const Gltf& g, int64_t idx) {
    const Json& a = g.doc["accessors"][(size_t)idx];
    if (a.type != Json::Object) fail(REINA_ERR_IO, "glTF: accessor " + std::to_string(idx) + " missing");
    if (a.has("sparse")) fail(REINA_ERR_IO, "glTF: sparse accessors are not supported");
    Accessor r;
    r.count = (size_t)a["count"].integer(0);
    r.ctype = (int)a["componentType"].integer(0);
    r.comps = type_comps(a["type"].string(""));
    r.normalized = a["normalized"].boolean(false);
    const int csize = ctype_size(r.ctype);
    if (!csize || !r.comps) fail(REINA_ERR_IO, "glTF: accessor " + std::to_string(idx) + " has an unsupported type");
    if (!a.has("bufferView")) fail(REINA_ERR_IO, "glTF: accessors without buffer views are not supported");
    const Json& v = g.doc["bufferViews"][(size_t)a["bufferView"].integer(-1)];
    const int64_t b = v["buffer"].integer(-1);
    if (b < 0 || (size_t)b >= g.buffers.size()) fail(REINA_ERR_IO, "glTF: buffer view references a missing buffer");
    const std::vector<uint8_t>& buf = g.buffers[(size_t)b];
    const size_t off = (size_t)v["byteOffset"].integer(0) + (size_t)a["byteOffset"].integer(0);
    const size_t elem = (size_t)csize * r.comps;
    r.stride = v.has("byteStride") ? (size_t)v["byteStride"].integer(0) : elem;
    if (r.stride < elem) fail(REINA_ERR_IO, "glTF: byteStride smaller than the element");
    const size_t view_end = (size_t)v["byteOffset"].integer(0) + (size_t)v["byteLength"].integer(0);
    if (r.count && (off + (r.count - 1) * r.stride + elem > view_end || view_end > buf.size()))
        fail(REINA_ERR_IO, "glTF: accessor " + std::to_string(idx) + " runs past its buffer");
    r.base = buf.data() + off;
    return r;
}

// column-major 4x4 products and TRS composition (glTF node transforms)
void mat_mul(const float a[16], const float b[16], float o[16]) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) {
            float s = 0.0f;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + rr] * b[c * 4 + k];
            r[c * 4 + rr] = s;
        }
    std::memcpy(o, r, sizeof(r));
}

void node_local(const Json& n, float m[16]) {
    if (n.has("matrix")) {
        for (int k = 0; k < 16; ++k) m[k] = (float)n["matrix"][(size_t)k].number(k % 5 == 0 ? 1.0 : 0.0);
        return;
    }
    const float tx = (float)n["translation"][0].number(0), ty = (float)n["translation"][1].number(0),
                tz = (float)n["translation"][2].number(0);
    const float qx = (float)n["rotation"][0].number(0), qy = (float)n["rotation"][1].number(0),
                qz = (float)n["rotation"][2].number(0), qw = (float)n["rotation"][3].number(1);
    const float sx = (float)n["scale"][0].number(1), sy = (float)n["scale"][1].number(1), sz = (float)n["scale"][2].number(1);
    const float R[9] = {1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy + qz * qw), 2 * (qx * qz - qy * qw),
                        2 * (qx * qy - qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz + qx * qw),
                        2 * (qx * qz + qy * qw), 2 * (qy * qz - qx * qw), 1 - 2 * (qx * qx + qy * qy)};
    const float s[3] = {sx, sy, sz};
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) m[c * 4 + r] = R[c * 3 + r] * s[c];
    m[3] = m[7] = m[11] = 0.0f;
    m[12] = tx; m[13] = ty; m[14] = tz; m[15] = 1.0f;
}

// Percent-decoding of a relative URI reference (RFC 3986 section 2.1).
std::string uri_path(const std::string& uri) {
    std::string out;
    for (size_t i = 0; i < uri.size(); ++i) {
        if (uri[i] == '%' && i + 2 < uri.size() && std::isxdigit((unsigned char)uri[i + 1]) &&
            std::isxdigit((unsigned char)uri[i + 2])) {
            out.push_back((char)std::stoi(uri.substr(i + 1, 2), nullptr, 16));
            i += 2;
        } else {
            out.push_back(uri[i]);
        }
    }
    return out;
}

// addTexturesToScene (gltfloader.cpp:283-340): every image of the asset becomes a scene texture, in image
// order, decoded from its bytes without a vertical flip (the parser loads external image files into
// memory, so every source reaches Scene::defineTexture(bytes)).  Returns the texture id per image; an
// image that cannot be decoded (a format other than PNG and sequential JPEG) gets -1, and the material references to it are
// counted as ignored.
std::vector<int32_t> gltf_images(const Gltf& g, const std::string& base_dir, Scene& scene) {
    const Json& imgs = g.doc["images"];
    std::vector<int32_t> ids(imgs.size(), -1);
    for (size_t i = 0; i < imgs.size(); ++i) {
        const Json& im = imgs[i];
        std::vector<uint8_t> bytes;
        if (im.has("uri")) {
            const std::string uri = im["uri"].string("");
            if (uri.rfind("data:", 0) == 0) {
                const size_t comma = uri.find(";base64,");
                if (comma == std::string::npos) fail(REINA_ERR_IO, "glTF: only base64 data URIs are supported");
                bytes = base64_decode(uri, comma + 8);
            } else {
                if (uri.find("://") != std::string::npos)
                    fail(REINA_ERR_IO, "Non-local URIs are not supported for texture loading");
                bytes = read_file(base_dir + "/" + uri_path(uri));
            }
        } else if (im.has("bufferView")) {
            const Json& v = g.doc["bufferViews"][(size_t)im["bufferView"].integer(-1)];
            const int64_t b = v["buffer"].integer(-1);
            if (b < 0 || (size_t)b >= g.buffers.size()) fail(REINA_ERR_IO, "glTF: image buffer view references a missing buffer");
            const std::vector<uint8_t>& buf = g.buffers[(size_t)b];
            const size_t off = (size_t)v["byteOffset"].integer(0), len = (size_t)v["byteLength"].integer(0);
            if (off > buf.size() || len > buf.size() - off) fail(REINA_ERR_IO, "glTF: image buffer view runs past its buffer");
            bytes.assign(buf.begin() + (ptrdiff_t)off, buf.begin() + (ptrdiff_t)(off + len));
        } else {
            continue;
        }
        try {
            ids[i] = (int32_t)scene.define_texture(decode_image(bytes.data(), bytes.size()));
        } catch (const Error& e) {
            if (e.code != REINA_ERR_IO) throw;
        }
    }
    return ids;
}

// Scene texture id of a material's texture reference ({"index": texture}); -1 (counted) when unresolved.
int32_t gltf_texture_ref(const Gltf& g, const Json& ref, const std::vector<int32_t>& image_ids, GltfLoadStats& st) {
    const Json& t = g.doc["textures"][(size_t)ref["index"].integer(-1)];
    const int64_t src = t["source"].integer(-1);
    if (t.type != Json::Object || src < 0 || (size_t)src >= image_ids.size() || image_ids[(size_t)src] < 0) {
        st.ignored_textures++;
        return -1;
    }
    return image_ids[(size_t)src];
}

// gltfloader.cpp:380-430: the default material is Disney with albedo 1, ior 1.5, interpolated normals;
// baseColorTexture -> texture_id, normalTexture -> normal_map_id.
reina_material gltf_material(const Gltf& g, int64_t mi, const std::vector<int32_t>& image_ids, GltfLoadStats& st) {
    reina_material m;
    std::memset(&m, 0, sizeof(m));
    m.material_idx = 3;
    m.texture_id = m.normal_map_id = m.bump_map_id = -1;
    for (int k = 0; k < 3; ++k) { m.albedo[k] = 1.0f; m.sheen_tint[k] = 1.0f; m.specular_tint[k] = 1.0f; }
    m.ior = 1.5f;
    m.interp_normals = 1;
    if (mi < 0) return m;
    const Json& j = g.doc["materials"][(size_t)mi];
    const Json& pbr = j["pbrMetallicRoughness"];
    const Json& ext = j["extensions"];
    float ef[3] = {(float)j["emissiveFactor"][0].number(0), (float)j["emissiveFactor"][1].number(0),
                   (float)j["emissiveFactor"][2].number(0)};
    const float strength = (float)ext["KHR_materials_emissive_strength"]["emissiveStrength"].number(1.0);
    if ((ef[0] > 0 || ef[1] > 0 || ef[2] > 0) && !j.has("emissiveTexture"))
        for (int k = 0; k < 3; ++k) m.emission[k] = ef[k] * strength;
    m.metallic = (float)pbr["metallicFactor"].number(1.0);
    m.roughness = std::fmax(std::fmin((float)pbr["roughnessFactor"].number(1.0), 0.7f), 0.1f);
    for (int k = 0; k < 3; ++k) m.albedo[k] = (float)pbr["baseColorFactor"][(size_t)k].number(1.0);
    m.cull_backface = j["doubleSided"].boolean(false) ? 0 : 1;
    m.ior = (float)ext["KHR_materials_ior"]["ior"].number(1.5);
    if (ext.has("KHR_materials_transmission")) {
        m.specular_transmission = (float)ext["KHR_materials_transmission"]["transmissionFactor"].number(0.0);
        m.cull_backface = 0;
    }
    if (pbr.has("baseColorTexture")) m.texture_id = gltf_texture_ref(g, pbr["baseColorTexture"], image_ids, st);
    if (j.has("normalTexture")) m.normal_map_id = gltf_texture_ref(g, j["normalTexture"], image_ids, st);
    return m;
}

}  // namespace

GltfLoadStats load_gltf_memory(const uint8_t* data, size_t size, const std::string& base_dir, Scene& scene) {
    Gltf g;
    std::vector<uint8_t> glb_bin;
    bool have_glb_bin = false;
    if (size >= 12 && std::memcmp(data, "glTF", 4) == 0) {   // GLB container
        uint32_t version, length;
        std::memcpy(&version, data + 4, 4);
        std::memcpy(&length, data + 8, 4);
        if (version != 2) fail(REINA_ERR_IO, "glTF: GLB version " + std::to_string(version) + " is not supported");
        if (length > size) fail(REINA_ERR_IO, "glTF: truncated GLB");
        size_t off = 12;
        bool have_json = false;
        while (off + 8 <= length) {
            uint32_t clen, ctype;
            std::memcpy(&clen, data + off, 4);
            std::memcpy(&ctype, data + off + 4, 4);
            if (off + 8 + (size_t)clen > length) fail(REINA_ERR_IO, "glTF: truncated GLB chunk");
            if (ctype == 0x4E4F534Au && !have_json) {
                g.doc = parse_json(reinterpret_cast<const char*>(data + off + 8), clen);
                have_json = true;
            } else if (ctype == 0x004E4942u && !have_glb_bin) {
                glb_bin.assign(data + off + 8, data + off + 8 + clen);
                have_glb_bin = true;
            }
            off += 8 + (size_t)((clen + 3) & ~3u);
        }
        if (!have_json) fail(REINA_ERR_IO, "glTF: GLB without a JSON chunk");
    } else {
        g.doc = parse_json(reinterpret_cast<const char*>(data), size);
    }
    const Json& bufs = g.doc["buffers"];
    for (size_t b = 0; b < bufs.size(); ++b) {
        const Json& bj = bufs[b];
        if (!bj.has("uri")) {
            if (b != 0 || !have_glb_bin) fail(REINA_ERR_IO, "glTF: buffer without a URI");
            g.buffers.push_back(glb_bin);
            continue;
        }
        const std::string uri = bj["uri"].string("");
        if (uri.rfind("data:", 0) == 0) {
            const size_t comma = uri.find(";base64,");
            if (comma == std::string::npos) fail(REINA_ERR_IO, "glTF: only base64 data URIs are supported");
            g.buffers.push_back(base64_decode(uri, comma + 8));
        } else {
            if (uri.find("://") != std::string::npos) fail(REINA_ERR_IO, "glTF: only local buffer files are supported");
            g.buffers.push_back(read_file(base_dir + "/" + uri));
        }
    }
    const Json& scenes = g.doc["scenes"];
    if (scenes.size() == 0) fail(REINA_ERR_IO, "No scenes supplied in gLTF file");
    const size_t scene_idx = (size_t)g.doc["scene"].integer(0);
    if (scene_idx >= scenes.size()) fail(REINA_ERR_IO, "glTF: default scene out of range");

    GltfLoadStats st;
    const std::vector<int32_t> image_ids = gltf_images(g, base_dir, scene);
    std::unordered_map<int64_t, std::vector<std::pair<uint32_t, int64_t>>> mesh_objects;   // mesh -> (object, material)
    auto define_mesh = [&](int64_t mi) -> const std::vector<std::pair<uint32_t, int64_t>>& {
        auto it = mesh_objects.find(mi);
        if (it != mesh_objects.end()) return it->second;
        std::vector<std::pair<uint32_t, int64_t>> objs;
        const Json& mesh = g.doc["meshes"][(size_t)mi];
        if (mesh.type != Json::Object) fail(REINA_ERR_IO, "glTF: node references a missing mesh");
        st.meshes++;
        const Json& prims = mesh["primitives"];
        for (size_t p = 0; p < prims.size(); ++p) {
            const Json& pj = prims[p];
            if (pj["mode"].integer(4) != 4) {   // triangles only
                st.skipped_primitives++;
                continue;
            }
            const Json& at = pj["attributes"];
            if (!at.has("POSITION")) fail(REINA_ERR_IO, "glTF: primitive without POSITION");
            if (!at.has("NORMAL")) fail(REINA_ERR_IO, "Meshes without vertex normals are not supported");
            const Accessor pa = accessor(g, at["POSITION"].integer(-1));
            const Accessor na = accessor(g, at["NORMAL"].integer(-1));
            if (pa.comps != 3 || na.comps != 3 || na.count != pa.count)
                fail(REINA_ERR_IO, "glTF: POSITION / NORMAL must be VEC3 of one count");
            const size_t nv = pa.count;
            ModelData md;
            std::vector<float> normals(3 * nv), uvs(2 * nv, 0.0f);
            md.vertices.resize(4 * nv);
            for (size_t v = 0; v < nv; ++v) {
                for (int k = 0; k < 3; ++k) {
                    md.vertices[4 * v + k] = pa.get(v, k);
                    normals[3 * v + k] = na.get(v, k);
                }
                md.vertices[4 * v + 3] = 1.0f;
            }
            if (at.has("TEXCOORD_0")) {
                const Accessor ta = accessor(g, at["TEXCOORD_0"].integer(-1));
                if (ta.comps != 2 || ta.count != nv) fail(REINA_ERR_IO, "glTF: TEXCOORD_0 must be VEC2 of the vertex count");
                for (size_t v = 0; v < nv; ++v) { uvs[2 * v] = ta.get(v, 0); uvs[2 * v + 1] = ta.get(v, 1); }
            }
            if (pj.has("indices")) {
                const Accessor ia = accessor(g, pj["indices"].integer(-1));
                if (ia.comps != 1 || (ia.ctype != 5121 && ia.ctype != 5123 && ia.ctype != 5125))
                    fail(REINA_ERR_IO, "glTF: indices must be unsigned scalars");
                md.indices.resize(ia.count);
                for (size_t i = 0; i < ia.count; ++i) {
                    md.indices[i] = ia.index(i);
                    if (md.indices[i] >= nv) fail(REINA_ERR_IO, "glTF: index out of range");
                }
            } else {   // non-indexed: one index per vertex
                md.indices.resize(nv);
                for (size_t i = 0; i < nv; ++i) md.indices[i] = (uint32_t)i;
            }
            md.indices.resize(md.indices.size() / 3 * 3);
            if (at.has("TANGENT")) {   // gltfloader.cpp:174-205: B = cross(N, T) * w (w = 1 for VEC3)
                const Accessor ta = accessor(g, at["TANGENT"].integer(-1));
                if ((ta.comps != 3 && ta.comps != 4) || ta.count != nv) fail(REINA_ERR_IO, "glTF: bad TANGENT accessor");
                md.tbns.resize(9 * nv);
                for (size_t v = 0; v < nv; ++v) {
                    float T[3] = {ta.get(v, 0), ta.get(v, 1), ta.get(v, 2)}, Nn[3] = {normals[3 * v], normals[3 * v + 1], normals[3 * v + 2]};
                    float B[3];
                    cross3(Nn, T, B);
                    const float w = ta.comps == 4 ? ta.get(v, 3) : 1.0f;
                    for (int k = 0; k < 3; ++k) {
                        md.tbns[9 * v + k] = T[k];
                        md.tbns[9 * v + 3 + k] = B[k] * w;
                        md.tbns[9 * v + 6 + k] = Nn[k];
                    }
                }
            } else {
                tangent_frames(md.vertices, normals, uvs, md.indices, md.tbns);
            }
            md.tbn_indices = md.indices;
            md.tex_coords = uvs;
            md.tex_indices = md.indices;
            if (md.indices.empty()) {
                st.skipped_primitives++;
                continue;
            }
            const uint32_t obj = scene.define_object(std::move(md));
            objs.emplace_back(obj, pj["material"].integer(-1));
            st.primitives++;
        }
        return mesh_objects.emplace(mi, std::move(objs)).first->second;
    };
    // depth-first over the default scene's node trees with world matrices
    const Json& roots = scenes[scene_idx]["nodes"];
    struct Item { int64_t node; float m[16]; int depth; };
    std::vector<Item> stack;
    for (size_t r = roots.size(); r-- > 0;) {
        Item it;
        it.node = roots[r].integer(-1);
        mat4_identity(it.m);
        it.depth = 0;
        stack.push_back(it);
    }
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        const Json& n = g.doc["nodes"][(size_t)it.node];
        if (n.type != Json::Object) fail(REINA_ERR_IO, "glTF: scene references a missing node");
        if (it.depth > 256) fail(REINA_ERR_IO, "glTF: node hierarchy too deep (cycle?)");
        float local[16], world[16];
        node_local(n, local);
        mat_mul(it.m, local, world);
        if (n.has("mesh")) {
            for (const auto& [obj, mat] : define_mesh(n["mesh"].integer(-1))) {
                const reina_material m = gltf_material(g, mat, image_ids, st);
                scene.add_instance(obj, world, m);
                st.instances++;
            }
        }
        const Json& ch = n["children"];
        for (size_t c = ch.size(); c-- > 0;) {
            Item ci;
            ci.node = ch[c].integer(-1);
            std::memcpy(ci.m, world, sizeof(world));
            ci.depth = it.depth + 1;
            stack.push_back(ci);
        }
    }
    return st;
}

GltfLoadStats load_gltf(const std::string& path, Scene& scene) {
    const std::vector<uint8_t> d = read_file(path);
    return load_gltf_memory(d.data(), d.size(), dir_of(path), scene);
}

}  // namespace rt
