// Seeded synthetic workloads: subdivided and noise-displaced icospheres, the ray sets of the ray-cast
// workload, and the camera matrices of src/graphics/Camera.cpp:10-11.  Only +, -, *, /, sqrt and floor
// are used where outputs must be identical on every host (compile with -ffp-contract=off).
#include "generators.h"

#include <cmath>
#include <cstring>
#include <unordered_map>

namespace rt {

uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double splitmix_unit(uint64_t& state) { return (double)(splitmix64(state) >> 11) * (1.0 / 9007199254740992.0); }

// Integer-lattice hash of (ix, iy, iz, seed) -> [-1, 1].
static double lattice(int64_t ix, int64_t iy, int64_t iz, uint64_t seed) {
    uint64_t h = seed * 0xD1B54A32D192ED03ull;
    h ^= (uint64_t)ix * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)iy * 0xC2B2AE3D27D4EB4Full;
    h ^= (uint64_t)iz * 0x165667B19E3779F9ull;
    uint64_t s = h;
    const uint64_t z = splitmix64(s);
    return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

static double smooth(double f) { return f * f * (3.0 - 2.0 * f); }

static double value_noise(double x, double y, double z, uint64_t seed) {
    const double fx0 = std::floor(x), fy0 = std::floor(y), fz0 = std::floor(z);
    const int64_t x0 = (int64_t)fx0, y0 = (int64_t)fy0, z0 = (int64_t)fz0;
    const double sx = smooth(x - fx0), sy = smooth(y - fy0), sz = smooth(z - fz0);
    double c[2][2][2];
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) c[i][j][k] = lattice(x0 + i, y0 + j, z0 + k, seed);
    auto lerp = [](double a, double b, double t) { return a + (b - a) * t; };
    const double x00 = lerp(c[0][0][0], c[1][0][0], sx), x10 = lerp(c[0][1][0], c[1][1][0], sx);
    const double x01 = lerp(c[0][0][1], c[1][0][1], sx), x11 = lerp(c[0][1][1], c[1][1][1], sx);
    const double y0v = lerp(x00, x10, sy), y1v = lerp(x01, x11, sy);
    return lerp(y0v, y1v, sz);
}

double fractal_noise3(double x, double y, double z, uint64_t seed) {
    // 3 octaves, base frequency 2, lacunarity 2, gain 0.5, normalized by the amplitude sum to [-1, 1].
    double sum = 0.0, amp = 1.0, freq = 2.0, norm = 0.0;
    for (int o = 0; o < 3; ++o) {
        sum += amp * value_noise(x * freq, y * freq, z * freq, seed + (uint64_t)o);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return sum / norm;
}

void icosphere_counts(uint32_t level, uint64_t& nv, uint64_t& nt) {
    uint64_t p = 1;
    for (uint32_t i = 0; i < level; ++i) p *= 4;
    nv = 10 * p + 2;
    nt = 20 * p;
}

// Unit icosahedron: 12 vertices (3 doubles each) and 20 outward-wound faces.
static void icosahedron(std::vector<double>& v, std::vector<uint32_t>& f) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    v = {-1, t, 0, 1, t, 0, -1, -t, 0, 1, -t, 0, 0, -1, t, 0, 1, t,
         0, -1, -t, 0, 1, -t, t, 0, -1, t, 0, 1, -t, 0, -1, -t, 0, 1};
    for (size_t i = 0; i < v.size(); i += 3) {
        const double l = std::sqrt(v[i] * v[i] + v[i + 1] * v[i + 1] + v[i + 2] * v[i + 2]);
        v[i] /= l; v[i + 1] /= l; v[i + 2] /= l;
    }
    f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
         3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
}

// Unit-sphere points -> vertices displaced radially to r = 1 + amplitude * noise (w = 1), plus the
// undisplaced directions as normals.
static void displace(const std::vector<double>& v, float amplitude, uint64_t seed, float* out_vertices, float* out_normals) {
    const size_t nv = v.size() / 3;
    for (size_t i = 0; i < nv; ++i) {
        const double x = v[3 * i], y = v[3 * i + 1], z = v[3 * i + 2];
        const double r = 1.0 + (double)amplitude * fractal_noise3(x, y, z, seed);
        out_vertices[4 * i + 0] = (float)(x * r);
        out_vertices[4 * i + 1] = (float)(y * r);
        out_vertices[4 * i + 2] = (float)(z * r);
        out_vertices[4 * i + 3] = 1.0f;
        if (out_normals) {
            out_normals[3 * i + 0] = (float)x;
            out_normals[3 * i + 1] = (float)y;
            out_normals[3 * i + 2] = (float)z;
        }
    }
}

void gen_icosphere(uint32_t level, float amplitude, uint64_t seed, float* out_vertices, uint32_t* out_indices,
                   float* out_normals) {
    std::vector<double> v;
    std::vector<uint32_t> f;
    icosahedron(v, f);
    for (uint32_t l = 0; l < level; ++l) {
        std::unordered_map<uint64_t, uint32_t> mid;
        mid.reserve(f.size());
        auto midpoint = [&](uint32_t a, uint32_t b) {
            const uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            double x = 0.5 * (v[3 * a] + v[3 * b]), y = 0.5 * (v[3 * a + 1] + v[3 * b + 1]), z = 0.5 * (v[3 * a + 2] + v[3 * b + 2]);
            const double len = std::sqrt(x * x + y * y + z * z);
            x /= len; y /= len; z /= len;
            const uint32_t id = (uint32_t)(v.size() / 3);
            v.push_back(x); v.push_back(y); v.push_back(z);
            mid.emplace(key, id);
            return id;
        };
        std::vector<uint32_t> nf;
        nf.reserve(f.size() * 4);
        for (size_t i = 0; i < f.size(); i += 3) {
            const uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
            const uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            const uint32_t tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), tri, tri + 12);
        }
        f.swap(nf);
    }
    displace(v, amplitude, seed, out_vertices, out_normals);
    std::memcpy(out_indices, f.data(), f.size() * sizeof(uint32_t));
}

void geodesic_counts(uint32_t frequency, uint64_t& nv, uint64_t& nt) {
    const uint64_t n = frequency;
    nv = 10 * n * n + 2;
    nt = 20 * n * n;
}

// Class-I geodesic sphere: every icosahedron face cut into a frequency x frequency triangular grid and
// projected to the unit sphere.  Vertices shared by faces (corners, then the frequency-1 interior points
// of each edge, then face interiors) are generated once, an edge's points always from its lower-indexed
// end, so neighbouring faces meet exactly.
void gen_geodesic(uint32_t frequency, float amplitude, uint64_t seed, float* out_vertices, uint32_t* out_indices,
                  float* out_normals) {
    const uint32_t n = frequency;
    std::vector<double> v;
    std::vector<uint32_t> f;
    icosahedron(v, f);
    const uint32_t inner = n - 1;   // interior points per edge
    std::unordered_map<uint64_t, uint32_t> edge_id;
    std::vector<uint32_t> edges;    // (lo, hi) pairs in id order
    for (size_t t = 0; t < f.size(); t += 3)
        for (int e = 0; e < 3; ++e) {
            const uint32_t a = f[t + e], b = f[t + (e + 1) % 3];
            const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
            if (edge_id.emplace((uint64_t)lo << 32 | hi, (uint32_t)(edges.size() / 2)).second) {
                edges.push_back(lo);
                edges.push_back(hi);
            }
        }
    auto push_point = [&](const double p[3]) {
        const double l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        v.push_back(p[0] / l); v.push_back(p[1] / l); v.push_back(p[2] / l);
    };
    for (size_t e = 0; e < edges.size(); e += 2) {
        const double* A = &v[3 * edges[e]];
        const double* B = &v[3 * edges[e + 1]];
        const double a0 = A[0], a1 = A[1], a2 = A[2], b0 = B[0], b1 = B[1], b2 = B[2];
        for (uint32_t k = 1; k <= inner; ++k) {
            const double t = (double)k / n;
            const double p[3] = {a0 + (b0 - a0) * t, a1 + (b1 - a1) * t, a2 + (b2 - a2) * t};
            push_point(p);
        }
    }
    const uint32_t face_base = (uint32_t)(v.size() / 3);
    const uint32_t per_face = n >= 2 ? (n - 1) * (n - 2) / 2 : 0;
    // vertex id of grid point (i, j) of face (A, B, C): A + (B - A) i/n + (C - A) j/n
    auto on_edge = [&](uint32_t a, uint32_t b, uint32_t k) {   // k of n steps from a towards b
        const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
        const uint32_t kk = a < b ? k : n - k;
        return 12 + edge_id.at((uint64_t)lo << 32 | hi) * inner + (kk - 1);
    };
    auto grid_id = [&](uint32_t face, uint32_t i, uint32_t j) -> uint32_t {
        const uint32_t A = f[3 * face], B = f[3 * face + 1], C = f[3 * face + 2];
        if (i == 0 && j == 0) return A;
        if (i == n) return B;
        if (j == n) return C;
        if (j == 0) return on_edge(A, B, i);
        if (i == 0) return on_edge(A, C, j);
        if (i + j == n) return on_edge(B, C, j);
        // interior: row j (1..n-2), column i (1..n-1-j)
        const uint32_t idx = (j - 1) * (n - 1) - (j - 1) * j / 2;   // points in rows 1..j-1
        return face_base + face * per_face + idx + (i - 1);
    };
    for (uint32_t face = 0; face < 20; ++face) {
        const double* A = &v[3 * f[3 * face]];
        const double* B = &v[3 * f[3 * face + 1]];
        const double* C = &v[3 * f[3 * face + 2]];
        const double a[3] = {A[0], A[1], A[2]}, b[3] = {B[0], B[1], B[2]}, c[3] = {C[0], C[1], C[2]};
        for (uint32_t j = 1; j + 1 < n; ++j)
            for (uint32_t i = 1; i + j < n; ++i) {
                const double s = (double)i / n, t = (double)j / n;
                const double p[3] = {a[0] + (b[0] - a[0]) * s + (c[0] - a[0]) * t, a[1] + (b[1] - a[1]) * s + (c[1] - a[1]) * t,
                                     a[2] + (b[2] - a[2]) * s + (c[2] - a[2]) * t};
                push_point(p);
            }
    }
    uint32_t* out = out_indices;
    for (uint32_t face = 0; face < 20; ++face)
        for (uint32_t j = 0; j < n; ++j)
            for (uint32_t i = 0; i + j < n; ++i) {
                *out++ = grid_id(face, i, j);
                *out++ = grid_id(face, i + 1, j);
                *out++ = grid_id(face, i, j + 1);
                if (i + j + 1 < n) {
                    *out++ = grid_id(face, i + 1, j);
                    *out++ = grid_id(face, i + 1, j + 1);
                    *out++ = grid_id(face, i, j + 1);
                }
            }
    displace(v, amplitude, seed, out_vertices, out_normals);
}

static void normalize3(double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
}

static void cross3(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}

// glm::perspective (right-handed, clip depth -1..1) and glm::lookAt, inverted.
void camera_matrices(const float pos[3], const float front[3], const float up[3], float fovy, float aspect,
                     float znear, float zfar, float inv_view[16], float inv_proj[16]) {
    double f[3] = {front[0], front[1], front[2]};
    normalize3(f);
    double u0[3] = {up[0], up[1], up[2]};
    double s[3];
    cross3(f, u0, s);
    normalize3(s);
    double u[3];
    cross3(s, f, u);
    // lookAt has rows s, u, -f; its inverse has those vectors as columns and the eye as translation.
    for (int r = 0; r < 3; ++r) {
        inv_view[0 * 4 + r] = (float)s[r];
        inv_view[1 * 4 + r] = (float)u[r];
        inv_view[2 * 4 + r] = (float)(-f[r]);
        inv_view[3 * 4 + r] = pos[r];
    }
    inv_view[3] = inv_view[7] = inv_view[11] = 0.0f;
    inv_view[15] = 1.0f;
    // perspective: P00 = 1/(aspect tan), P11 = 1/tan, P22 = -(f+n)/(f-n), P23 = -1, P32 = -2fn/(f-n).
    const double th = std::tan((double)fovy / 2.0);
    const double p00 = 1.0 / ((double)aspect * th), p11 = 1.0 / th;
    const double p22 = -((double)zfar + znear) / ((double)zfar - znear);
    const double p32 = -(2.0 * zfar * znear) / ((double)zfar - znear);
    // inverse of [[p00,0,0,0],[0,p11,0,0],[0,0,p22,p32],[0,0,-1,0]] (row-major math form)
    for (int i = 0; i < 16; ++i) inv_proj[i] = 0.0f;
    inv_proj[0 * 4 + 0] = (float)(1.0 / p00);
    inv_proj[1 * 4 + 1] = (float)(1.0 / p11);
    inv_proj[2 * 4 + 3] = (float)(1.0 / p32);     // column 2, row 3
    inv_proj[3 * 4 + 2] = -1.0f;                  // column 3, row 2
    inv_proj[3 * 4 + 3] = (float)(p22 / p32);     // column 3, row 3
}

void gen_raycast_rays(uint32_t width, uint32_t height, const float cam_pos[3], const float cam_target[3],
                      float fovy_degrees, uint64_t n_random, const float box_min[3], const float box_max[3],
                      uint64_t seed, Ray* out) {
    double f[3] = {(double)cam_target[0] - cam_pos[0], (double)cam_target[1] - cam_pos[1], (double)cam_target[2] - cam_pos[2]};
    normalize3(f);
    double up[3] = {0.0, 1.0, 0.0};
    double s[3];
    cross3(f, up, s);
    normalize3(s);
    double u[3];
    cross3(s, f, u);
    const double th = std::tan((double)fovy_degrees * 3.14159265358979323846 / 360.0);
    const double aspect = (double)width / (double)height;
    uint64_t k = 0;
    for (uint32_t y = 0; y < height; ++y) {
        for (uint32_t x = 0; x < width; ++x, ++k) {
            const double nx = (2.0 * (x + 0.5) / width - 1.0) * th * aspect;
            const double ny = (1.0 - 2.0 * (y + 0.5) / height) * th;
            double d[3];
            for (int c = 0; c < 3; ++c) d[c] = f[c] + nx * s[c] + ny * u[c];
            normalize3(d);
            Ray& r = out[k];
            r.ox = cam_pos[0]; r.oy = cam_pos[1]; r.oz = cam_pos[2]; r.tmin = 0.0f;
            r.dx = (float)d[0]; r.dy = (float)d[1]; r.dz = (float)d[2]; r.tmax = 1e4f;
        }
    }
    uint64_t st = seed ^ 0x5851F42D4C957F2Dull;
    for (uint64_t i = 0; i < n_random; ++i, ++k) {
        double o[3];
        for (int c = 0; c < 3; ++c) o[c] = box_min[c] + ((double)box_max[c] - box_min[c]) * splitmix_unit(st);
        double d[3];
        for (;;) {
            for (int c = 0; c < 3; ++c) d[c] = 2.0 * splitmix_unit(st) - 1.0;
            const double l2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (l2 > 1e-6 && l2 <= 1.0) break;
        }
        normalize3(d);
        Ray& r = out[k];
        r.ox = (float)o[0]; r.oy = (float)o[1]; r.oz = (float)o[2]; r.tmin = 0.0f;
        r.dx = (float)d[0]; r.dy = (float)d[1]; r.dz = (float)d[2]; r.tmax = 1e4f;
    }
}

}  // namespace rt
