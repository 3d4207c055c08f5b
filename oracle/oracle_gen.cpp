// ORACLE — test infrastructure only.  The synthetic ray-cast workload restated on the host, so that the
// timed CPU arm of bench.py (`--impl reference`) builds its triangles and rays without loading the
// product library: the level-L icosphere (icosahedron, 4-way midpoint subdivision with new vertices in
// first-use order, radial displacement r = 1 + amplitude * 3-octave value noise) and the ray set
// (width x height pinhole camera through pixel centres, then n_random rays with origins uniform in a box
// and directions uniform on the sphere by rejection), both from SplitMix64 streams.  tests/test_oracle.py
// checks both against the product's generators bit for bit.  Built with -ffp-contract=off; only + - * /,
// sqrt, floor and tan are used.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

namespace {

struct Mix {
    uint64_t s;
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// Lattice value in [-1, 1] of integer point (i, j, k) for `seed`.
double corner(int64_t i, int64_t j, int64_t k, uint64_t seed) {
    Mix m{seed * 0xD1B54A32D192ED03ull ^ (uint64_t)i * 0x9E3779B97F4A7C15ull ^ (uint64_t)j * 0xC2B2AE3D27D4EB4Full ^
          (uint64_t)k * 0x165667B19E3779F9ull};
    return (double)(m.next() >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

double fade(double t) { return t * t * (3.0 - 2.0 * t); }
double mixd(double a, double b, double t) { return a + (b - a) * t; }

// Trilinear value noise with smoothstep weights.
double noise(double x, double y, double z, uint64_t seed) {
    const double bx = std::floor(x), by = std::floor(y), bz = std::floor(z);
    const int64_t ix = (int64_t)bx, iy = (int64_t)by, iz = (int64_t)bz;
    const double wx = fade(x - bx), wy = fade(y - by), wz = fade(z - bz);
    double zl[2];
    for (int dz = 0; dz < 2; ++dz) {
        const double a = mixd(corner(ix, iy, iz + dz, seed), corner(ix + 1, iy, iz + dz, seed), wx);
        const double b = mixd(corner(ix, iy + 1, iz + dz, seed), corner(ix + 1, iy + 1, iz + dz, seed), wx);
        zl[dz] = mixd(a, b, wy);
    }
    return mixd(zl[0], zl[1], wz);
}

// Octaves at frequencies 2, 4, 8 with weights 1, 1/2, 1/4 (seeds seed, seed+1, seed+2), over the weight sum.
double octaves(double x, double y, double z, uint64_t seed) {
    double total = 0.0, weights = 0.0, w = 1.0, f = 2.0;
    for (uint64_t o = 0; o < 3; ++o) {
        total += w * noise(x * f, y * f, z * f, seed + o);
        weights += w;
        w *= 0.5;
        f *= 2.0;
    }
    return total / weights;
}

struct P3 {
    double x, y, z;
};

P3 unit(P3 p) {
    const double n = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
    return P3{p.x / n, p.y / n, p.z / n};
}

P3 cross(const P3& a, const P3& b) { return P3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }

}  // namespace

extern "C" {

void oracle_icosphere_counts(uint32_t level, uint64_t* nv, uint64_t* nt) {
    const uint64_t q = 1ull << (2 * level);
    *nv = 10 * q + 2;
    *nt = 20 * q;
}

// Vertices (x, y, z, 1) and triangle indices of the displaced level-`level` icosphere.
void oracle_gen_icosphere(uint32_t level, float amplitude, uint64_t seed, float* v4, uint32_t* idx) {
    const double g = (1.0 + std::sqrt(5.0)) / 2.0;
    const double base[12][3] = {{-1, g, 0}, {1, g, 0}, {-1, -g, 0}, {1, -g, 0}, {0, -1, g}, {0, 1, g},
                                {0, -1, -g}, {0, 1, -g}, {g, 0, -1}, {g, 0, 1}, {-g, 0, -1}, {-g, 0, 1}};
    std::vector<P3> pts;
    for (const auto& b : base) pts.push_back(unit(P3{b[0], b[1], b[2]}));
    std::vector<uint32_t> tri = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                                 11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                                 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (uint32_t l = 0; l < level; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> edge;   // undirected edge -> its midpoint vertex
        auto mid = [&](uint32_t a, uint32_t b) -> uint32_t {
            const std::pair<uint32_t, uint32_t> e = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
            const auto f = edge.find(e);
            if (f != edge.end()) return f->second;
            const P3 m = unit(P3{0.5 * (pts[a].x + pts[b].x), 0.5 * (pts[a].y + pts[b].y), 0.5 * (pts[a].z + pts[b].z)});
            pts.push_back(m);
            const uint32_t id = (uint32_t)pts.size() - 1;
            edge[e] = id;
            return id;
        };
        std::vector<uint32_t> out;
        out.reserve(tri.size() * 4);
        for (size_t t = 0; t < tri.size(); t += 3) {
            const uint32_t a = tri[t], b = tri[t + 1], c = tri[t + 2];
            const uint32_t ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
            for (uint32_t x : {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca}) out.push_back(x);
        }
        tri.swap(out);
    }
    for (size_t i = 0; i < pts.size(); ++i) {
        const P3 p = pts[i];
        const double r = 1.0 + (double)amplitude * octaves(p.x, p.y, p.z, seed);
        v4[4 * i + 0] = (float)(p.x * r);
        v4[4 * i + 1] = (float)(p.y * r);
        v4[4 * i + 2] = (float)(p.z * r);
        v4[4 * i + 3] = 1.0f;
    }
    std::memcpy(idx, tri.data(), tri.size() * sizeof(uint32_t));
}

// Rays (origin, tmin, direction, tmax as 8 floats): the camera's width x height rays (row by row, top row
// first), then the n_random box rays.
void oracle_gen_rays(uint32_t width, uint32_t height, const float* cam_pos, const float* cam_target, float fovy_degrees,
                     uint64_t n_random, const float* box_min, const float* box_max, uint64_t seed, float* out) {
    const P3 fwd = unit(P3{(double)cam_target[0] - cam_pos[0], (double)cam_target[1] - cam_pos[1],
                           (double)cam_target[2] - cam_pos[2]});
    const P3 right = unit(cross(fwd, P3{0.0, 1.0, 0.0}));
    const P3 up = cross(right, fwd);
    const double half = std::tan((double)fovy_degrees * 3.14159265358979323846 / 360.0);
    const double aspect = (double)width / (double)height;
    float* o = out;
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x, o += 8) {
            const double px = (2.0 * (x + 0.5) / width - 1.0) * half * aspect;
            const double py = (1.0 - 2.0 * (y + 0.5) / height) * half;
            const P3 d = unit(P3{fwd.x + px * right.x + py * up.x, fwd.y + px * right.y + py * up.y,
                                 fwd.z + px * right.z + py * up.z});
            const float r[8] = {cam_pos[0], cam_pos[1], cam_pos[2], 0.0f, (float)d.x, (float)d.y, (float)d.z, 1e4f};
            std::memcpy(o, r, sizeof(r));
        }
    Mix m{seed ^ 0x5851F42D4C957F2Dull};
    for (uint64_t i = 0; i < n_random; ++i, o += 8) {
        double org[3];
        for (int c = 0; c < 3; ++c) org[c] = box_min[c] + ((double)box_max[c] - box_min[c]) * m.unit();
        P3 d;
        for (;;) {
            d.x = 2.0 * m.unit() - 1.0;
            d.y = 2.0 * m.unit() - 1.0;
            d.z = 2.0 * m.unit() - 1.0;
            const double q = d.x * d.x + d.y * d.y + d.z * d.z;
            if (q > 1e-6 && q <= 1.0) break;
        }
        d = unit(d);
        const float r[8] = {(float)org[0], (float)org[1], (float)org[2], 0.0f, (float)d.x, (float)d.y, (float)d.z, 1e4f};
        std::memcpy(o, r, sizeof(r));
    }
}

}  // extern "C"
