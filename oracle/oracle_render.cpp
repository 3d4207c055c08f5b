// ORACLE — test infrastructure only (see oracle_common.h).
//
// CPU restatement of the reference's per-pixel megakernel (shaders/raytrace/raytrace.rgen.glsl), its hit
// reconstruction (closestHitCommon.h.glsl:52-148), the four closest-hit shaders (lambertian, metal,
// dielectric, disney .rchit.glsl), the sky miss shader (raytrace.rmiss.glsl:10-19), next-event estimation
// (nee.h.glsl, rgen directLight :43-95) and the emissive CDF construction (src/scene/Instance.cpp:15-53),
// in float or double precision, over the oracle's own scene representation and BVH.
//
// Integrator modes:
//   reina   — faithful: skipNEE = true (raytrace.rgen.glsl:146), per-pixel RNG seed
//             (sampleBatch*H + y)*W + x (:259) carried across the pixel's samples, and the payload's
//             accumulatedDistance carried across samples (it is never reset in the raygen shader; the
//             first sample of a launch starts from 0).
//   nee_mis — NEE on for Lambertian (0) and Disney (3) hits as the commented rule at :145 enables, with
//             power-heuristic MIS pairing each strategy with the other's pdf for the same direction: NEE
//             at vertex k is weighted against the BSDF pdf of the light direction, and emission found by
//             the BSDF ray from vertex k-1 against the light pdf of that point seen from k-1.  Each
//             (pixel, sample) path gets its own RNG seed hash(pixel, sample, seed).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "oracle_bsdf.h"
#include "oracle_common.h"

namespace oracle {

// Field-for-field copy of the C ABI's reina_material (src/scene/Scene.h:21-46).
struct OMaterial {
    uint32_t material_idx;
    int32_t texture_id, normal_map_id, bump_map_id;
    float albedo[3], emission[3];
    float roughness, ior;
    uint32_t interp_normals;
    float absorption;
    uint32_t cull_backface;
    float anisotropic, subsurface, clearcoat_gloss;
    float sheen_tint[3], specular_tint[3];
    float metallic, clearcoat, specular_transmission, sheen;
};

// polyglot/raytrace.h:43-54
struct OPush {
    float invView[16], invProjection[16];
    uint32_t sampleBatch;
    float totalEmissiveWeight, focusDist, defocusMultiplier, directClamp, indirectClamp;
    uint32_t samplesPerPixel, maxBounces;
};

struct ORenderOptions {
    uint32_t mode;          // 0 reina, 1 nee_mis
    uint32_t seed;
    uint32_t env_mode;      // 0 sky gradient (raytrace.rmiss.glsl), 1 constant colour
    float env_color[3];
    uint32_t x0, y0, x1, y1;   // pixel window to render (x1/y1 exclusive)
};

struct OObject {
    std::vector<float> v;        // 4 per vertex
    std::vector<uint32_t> idx;
    std::vector<float> tbn;      // 9 per entry (columns T, B, N)
    std::vector<uint32_t> tbn_idx;
    std::vector<float> uv;       // 2 per entry
    std::vector<uint32_t> uv_idx;   // 3 per triangle (0xFFFFFFFF: corner without UV)
};

// An RGBA8 texture, rows top to bottom (row 0 at v = 0), texel = r | g << 8 | b << 16 | a << 24.
struct OTexture {
    uint32_t w = 0, h = 0;
    std::vector<uint32_t> texels;
};

struct OInstance {
    uint32_t obj = 0;
    float T[16];
    std::vector<OMaterial> mats;
    std::vector<uint32_t> face_mat;
    uint32_t first_prim = 0;
    bool emissive = false;
    float weight = 0, area = 0;
    std::vector<float> cdf;
    uint32_t cdf_start = 0, cdf_end = 0;
};

struct OScene {
    std::vector<OObject> objects;
    std::vector<OInstance> instances;
    std::vector<float> world;           // 9 per global triangle
    std::vector<uint32_t> prim_inst;
    void* bvh = nullptr;
    std::vector<uint32_t> emissive;     // instance index per emissive position
    std::vector<float> cdf_instances, cdf_triangles;
    float total_weight = 0;
    std::vector<OTexture> textures;
};

}  // namespace oracle

extern "C" {
void* oracle_bvh_build(const float* tris9, uint64_t n);
void oracle_bvh_destroy(void* h);
}

namespace oracle {

// Declared in oracle_trace.cpp.
template <class T> struct BestHit;
struct Bvh;

// Float-mode closest hit with reported t/u/v refined in double (what the ray-cast API reports), or the
// double-mode closest hit; any-hit for shadow rays.
int trace_closest_f(void* bvh, const RayRec& r, uint32_t& prim, double& t, double& u, double& v, int precision);
bool trace_occluded(void* bvh, const RayRec& r, int precision);

template <class T>
struct Ctx {
    const OScene& s;
    const OPush& pc;
    const ORenderOptions& opt;
    int precision;
};

template <class T>
inline Vec3<T> load3(const float* p) { return Vec3<T>((T)p[0], (T)p[1], (T)p[2]); }

template <class T>
inline Vec3<T> xform_point(const float* M, Vec3<T> p) {   // column-major mat4 * vec4(p, 1)
    Vec3<T> r;
    for (int k = 0; k < 3; ++k) r[k] = (T)M[0 * 4 + k] * p.x + (T)M[1 * 4 + k] * p.y + (T)M[2 * 4 + k] * p.z + (T)M[3 * 4 + k];
    return r;
}
template <class T>
inline Vec3<T> xform_dir3(const float* M, Vec3<T> p) {   // mat3(M) * p
    Vec3<T> r;
    for (int k = 0; k < 3; ++k) r[k] = (T)M[0 * 4 + k] * p.x + (T)M[1 * 4 + k] * p.y + (T)M[2 * 4 + k] * p.z;
    return r;
}

template <class T>
struct HitInfo {
    Vec3<T> worldPosition, worldNormal, worldNormalGeometry;
    bool frontFace;
    Mat3<T> tbn;
    T uv[2];
};

// closestHitCommon.h.glsl:52-148.  UV: barycentric blend of the corner texture coordinates, (0, 0) for a
// model without them; a corner whose texture index is 0xFFFFFFFF contributes (0, 0).
template <class T>
HitInfo<T> getObjectHitInfo(const OScene& s, uint32_t prim, T bu, T bv, Vec3<T> rayDir) {
    const OInstance& inst = s.instances[s.prim_inst[prim]];
    const OObject& o = s.objects[inst.obj];
    const OMaterial& m = inst.mats[inst.face_mat.empty() ? 0 : inst.face_mat[prim - inst.first_prim]];
    const uint32_t lp = prim - inst.first_prim;
    const uint32_t i0 = o.idx[3 * lp], i1 = o.idx[3 * lp + 1], i2 = o.idx[3 * lp + 2];
    const Vec3<T> v0 = load3<T>(&o.v[4 * i0]), v1 = load3<T>(&o.v[4 * i1]), v2 = load3<T>(&o.v[4 * i2]);
    const T b0 = (T)1 - bu - bv;
    HitInfo<T> h;
    const Vec3<T> objPos = v0 * b0 + v1 * bu + v2 * bv;
    h.worldPosition = xform_point(inst.T, objPos);
    h.uv[0] = h.uv[1] = (T)0;
    if (!o.uv.empty() && !o.uv_idx.empty()) {
        T c[3][2];
        for (int k = 0; k < 3; ++k) {
            const uint32_t t = o.uv_idx[3 * lp + k];
            c[k][0] = t == 0xFFFFFFFFu ? (T)0 : (T)o.uv[2ull * t];
            c[k][1] = t == 0xFFFFFFFFu ? (T)0 : (T)o.uv[2ull * t + 1];
        }
        for (int a = 0; a < 2; ++a) h.uv[a] = c[0][a] * b0 + c[1][a] * bu + c[2][a] * bv;
    }
    const Vec3<T> ng = normalize(cross(v1 - v0, v2 - v0));
    const bool have_tbn = !o.tbn_idx.empty();
    Vec3<T> on = ng;
    Mat3<T> t0, t1, t2;
    if (have_tbn) {
        auto M = [&](uint32_t k) {
            const float* q = &o.tbn[9ull * o.tbn_idx[3 * lp + k]];
            return Mat3<T>{load3<T>(q), load3<T>(q + 3), load3<T>(q + 6)};
        };
        t0 = M(0); t1 = M(1); t2 = M(2);
        if (m.interp_normals) {
            const Vec3<T> n0 = normalize(t0.c2), n1 = normalize(t1.c2), n2 = normalize(t2.c2);
            on = normalize(n0 * b0 + n1 * bu + n2 * bv);
        }
    } else {
        // no TBN data: tangent frame (1,0,0), (0,1,0) and the geometric normal at every vertex
        t0.c0 = t1.c0 = t2.c0 = Vec3<T>((T)1, (T)0, (T)0);
        t0.c1 = t1.c1 = t2.c1 = Vec3<T>((T)0, (T)1, (T)0);
        t0.c2 = t1.c2 = t2.c2 = ng;
    }
    h.worldNormal = normalize(xform_dir3(inst.T, on));
    h.worldNormalGeometry = normalize(xform_dir3(inst.T, ng));
    h.frontFace = dot(rayDir, h.worldNormalGeometry) < (T)0;
    h.worldNormal = faceforward(h.worldNormal, rayDir, h.worldNormalGeometry);
    h.worldNormalGeometry = faceforward(h.worldNormalGeometry, rayDir, h.worldNormalGeometry);
    const Vec3<T> tangent = normalize(t0.c0 * b0 + t1.c0 * bu + t2.c0 * bv);
    const Vec3<T> bitangent = normalize(t0.c1 * b0 + t1.c1 * bu + t2.c1 * bv);
    const Vec3<T> normal = normalize(t0.c2 * b0 + t1.c2 * bu + t2.c2 * bv);
    // N = transpose(inverse(mat3(M))) = cofactor(M) / det(M)
    auto Mrc = [&](int r, int c) { return (T)inst.T[c * 4 + r]; };
    T cof[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
            cof[r][c] = Mrc(r1, c1) * Mrc(r2, c2) - Mrc(r1, c2) * Mrc(r2, c1);
        }
    const T det = Mrc(0, 0) * cof[0][0] + Mrc(0, 1) * cof[0][1] + Mrc(0, 2) * cof[0][2];
    Vec3<T> nN;
    for (int r = 0; r < 3; ++r) nN[r] = (cof[r][0] * normal.x + cof[r][1] * normal.y + cof[r][2] * normal.z) / det;
    Vec3<T> wT = normalize(xform_dir3(inst.T, tangent));
    Vec3<T> wB = normalize(xform_dir3(inst.T, bitangent));
    Vec3<T> wN = normalize(nN);
    wT = normalize(wT - wN * dot(wN, wT));
    wB = normalize(wB - wN * dot(wN, wB));
    wB = wB * (T)-1;
    wN = wN * (h.frontFace ? (T)1 : (T)-1);
    h.tbn = Mat3<T>{wT, wB, wN};
    return h;
}

// ---- textures (texutils.h.glsl, the sampler of src/tools/vktools.cpp:765-780) ----------------------

// One axis of bilinear addressing with REPEAT wrapping: coordinate c * size - 0.5, texels floor() and
// floor() + 1 modulo the size, weight frac(); non-finite coordinates address texel 0 with weight 0.
template <class T>
void tex_axis(T c, uint32_t size, uint32_t& i0, uint32_t& i1, T& w) {
    const T fs = (T)size;
    T x = c * fs - (T)0.5;
    if (!(std::fabs(x) <= (T)3.0e38)) x = 0;
    const T fx = std::floor(x);
    w = x - fx;
    T r = std::fmod(fx, fs);
    if (r < (T)0) r = r + fs;
    i0 = (uint32_t)r;
    i1 = i0 + 1u == size ? 0u : i0 + 1u;
}

// texture(sampler2D, uv) at level 0 on R8G8B8A8_UNORM texels: the four texels' 8-bit values blended with
// the bilinear weights, then divided by 255.
template <class T>
void tex_sample(const OScene& s, int id, T u, T v, T out[4]) {
    const OTexture& t = s.textures[(size_t)id];
    uint32_t x0, x1, y0, y1;
    T a, b;
    tex_axis(u, t.w, x0, x1, a);
    tex_axis(v, t.h, y0, y1, b);
    const uint32_t c00 = t.texels[(size_t)y0 * t.w + x0], c10 = t.texels[(size_t)y0 * t.w + x1];
    const uint32_t c01 = t.texels[(size_t)y1 * t.w + x0], c11 = t.texels[(size_t)y1 * t.w + x1];
    const T na = (T)1 - a, nb = (T)1 - b;
    const T w00 = na * nb, w10 = a * nb, w01 = na * b, w11 = a * b;
    for (int k = 0; k < 4; ++k) {
        const int sh = 8 * k;
        T acc = w00 * (T)((c00 >> sh) & 255u);
        acc = acc + w10 * (T)((c10 >> sh) & 255u);
        acc = acc + w01 * (T)((c01 >> sh) & 255u);
        acc = acc + w11 * (T)((c11 >> sh) & 255u);
        out[k] = acc / (T)255;
    }
}

// texutils.h.glsl:4-45 bumpMapping (parallax search of the height map's red channel).
template <class T>
void bumpMapping(const OScene& s, int id, T uv[2], Vec3<T> rayIn, const Mat3<T>& tbn) {
    const T heightScale = (T)0.2, minLayers = (T)64, maxLayers = (T)512;
    const Vec3<T> V = normalize(mulT(tbn, -rayIn));
    if (V.z <= (T)0) return;
    const T numLayers = mixs(maxLayers, minLayers, std::fmin(std::fmax(V.z, (T)0), (T)1));
    const T layerDepth = (T)1 / numLayers;
    const T P[2] = {V.x / V.z * heightScale, V.y / V.z * heightScale};
    const T d[2] = {P[0] / numLayers, P[1] / numLayers};
    T cur[2] = {uv[0], uv[1]};
    T depthSum = 0;
    T tex[4];
    tex_sample(s, id, cur[0], cur[1], tex);
    T h = tex[0] * heightScale;
    for (int it = 0; depthSum < h && it < 1024; ++it) {
        cur[0] = cur[0] - d[0];
        cur[1] = cur[1] - d[1];
        depthSum = depthSum + layerDepth;
        tex_sample(s, id, cur[0], cur[1], tex);
        h = tex[0] * heightScale;
    }
    const T prev[2] = {cur[0] + d[0], cur[1] + d[1]};
    tex_sample(s, id, prev[0], prev[1], tex);
    const T hPrev = tex[0] * heightScale;
    const T sumPrev = depthSum - layerDepth;
    const T after = h - depthSum;
    const T before = hPrev - sumPrev;
    const T weight = after / (after - before);
    uv[0] = mixs(prev[0], cur[0], weight);
    uv[1] = mixs(prev[1], cur[1], weight);
}

// The texture stage of the closest-hit shaders (lambertian.rchit.glsl:20-58, metal.rchit.glsl:18-50,
// dielectric.rchit.glsl:54-73, disney.rchit.glsl:19-72): uv = mod(uv, 1), bump mapping, the
// out-of-[0,1] skip (uv_check), the normal map, and the albedo texture with its alpha test (alpha_test).
// Returns false when the hit is skipped.
template <class T>
bool apply_textures(const OScene& s, const HitInfo<T>& hit, const OMaterial& m, Vec3<T> rayDir, uint32_t& rng,
                    bool uv_check, bool alpha_test, Vec3<T>& n, Vec3<T>& albedo) {
    n = hit.worldNormal;
    albedo = load3<T>(m.albedo);
    if (m.texture_id < 0 && m.normal_map_id < 0 && m.bump_map_id < 0) return true;
    T uv[2] = {hit.uv[0] - std::floor(hit.uv[0]), hit.uv[1] - std::floor(hit.uv[1])};
    if (m.bump_map_id >= 0) bumpMapping(s, m.bump_map_id, uv, normalize(rayDir), hit.tbn);
    if (uv_check && (uv[0] < (T)0 || uv[0] > (T)1 || uv[1] < (T)0 || uv[1] > (T)1)) return false;
    T tex[4];
    if (m.normal_map_id >= 0) {
        tex_sample(s, m.normal_map_id, uv[0], uv[1], tex);
        Vec3<T> tn(tex[0] * (T)2 - (T)1, tex[1] * (T)2 - (T)1, tex[2] * (T)2 - (T)1);
        tn.y = tn.y * (T)-1;
        n = normalize(mul(hit.tbn, tn));
    }
    if (m.texture_id >= 0) {
        tex_sample(s, m.texture_id, uv[0], uv[1], tex);
        if (alpha_test && tex[3] < (T)0.999 && rng_random<T>(rng) > tex[3]) return false;
        albedo = albedo * Vec3<T>(tex[0], tex[1], tex[2]);
    }
    return true;
}

// Per-path payload (shaderCommon.h.glsl:18-36), the fields the raygen loop reads.
template <class T>
struct Payload {
    Vec3<T> albedo, color, rayOrigin, rayDirection, emission, surfaceNormal;
    uint32_t rng = 0;
    bool rayHitSky = false, skip = false, insideDielectric = false, didRefract = false;
    uint32_t materialID = 0;
    T pdf = 0, accumulatedDistance = 0, eta = 0;
    Mat3<T> tbn;
    const OMaterial* props = nullptr;
    uint32_t prim = kMiss;
};

template <class T>
DisneyParams<T> disney_params(const OMaterial& m, Vec3<T> albedo) {
    DisneyParams<T> p;
    p.base = albedo;
    p.specTint = load3<T>(m.specular_tint);
    p.sheenTint = load3<T>(m.sheen_tint);
    p.aniso = (T)m.anisotropic;
    p.rough = (T)m.roughness;
    p.subsurface = (T)m.subsurface;
    p.ccGloss = (T)m.clearcoat_gloss;
    p.metallic = (T)m.metallic;
    p.clearcoat = (T)m.clearcoat;
    p.specTrans = (T)m.specular_transmission;
    p.sheen = (T)m.sheen;
    return p;
}

// traceRayEXT + the hit/miss shader that runs for it.
template <class T>
void trace_and_shade(const Ctx<T>& c, Vec3<T> org, Vec3<T> dir, Payload<T>& pld) {
    RayRec r{(float)org.x, (float)org.y, (float)org.z, 0.0f, (float)dir.x, (float)dir.y, (float)dir.z, 10000.0f};
    uint32_t prim;
    double ht, hu, hv;
    trace_closest_f(c.s.bvh, r, prim, ht, hu, hv, c.precision);
    pld.prim = prim;
    if (prim == kMiss) {   // raytrace.rmiss.glsl:10-19
        if (c.opt.env_mode == 1) {
            pld.color = load3<T>(c.opt.env_color);
        } else {
            const T y = normalize(dir).y;
            const T t = (T)0.5 * (y + (T)1);
            pld.color = mixv(Vec3<T>((T)0.1, (T)0.1, (T)0.1), Vec3<T>((T)0.4, (T)1.7, (T)2), t) * (T)0.07;
        }
        pld.albedo = pld.color;
        pld.rayHitSky = true;
        pld.skip = false;
        return;
    }
    const OInstance& inst = c.s.instances[c.s.prim_inst[prim]];
    const OMaterial& m = inst.mats[inst.face_mat.empty() ? 0 : inst.face_mat[prim - inst.first_prim]];
    const HitInfo<T> hit = getObjectHitInfo<T>(c.s, prim, (T)hu, (T)hv, dir);
    auto do_skip = [&]() {   // closestHitCommon.h.glsl:185-193
        pld.rayOrigin = offsetAlongNormal(hit.worldPosition, -hit.worldNormal);
        pld.rayDirection = dir;
        pld.rayHitSky = false;
        pld.skip = true;
    };
    Vec3<T> worldNormal, texAlbedo;
    if (m.material_idx == 0) {   // lambertian.rchit.glsl:11-78
        if (m.cull_backface && !hit.frontFace) { do_skip(); return; }
        if (!apply_textures(c.s, hit, m, dir, pld.rng, true, true, worldNormal, texAlbedo)) { do_skip(); return; }
        pld.color = texAlbedo;
        pld.albedo = pld.color;
        pld.emission = load3<T>(m.emission);
        pld.rayOrigin = offsetAlongNormal(hit.worldPosition, hit.worldNormalGeometry);
        pld.rayDirection = diffuseReflection<T>(worldNormal, pld.rng);
        pld.rayHitSky = false;
        pld.skip = false;
        pld.insideDielectric = false;
        pld.materialID = 0;
        pld.surfaceNormal = worldNormal;
        pld.pdf = pdfLambertian(pld.surfaceNormal, pld.rayDirection);
        pld.tbn = hit.tbn;
        pld.props = &m;
        pld.didRefract = false;
        pld.eta = 0;
        pld.accumulatedDistance = 0;
    } else if (m.material_idx == 1) {   // metal.rchit.glsl:7-70
        if (m.cull_backface && !hit.frontFace) { do_skip(); return; }
        if (!apply_textures(c.s, hit, m, dir, pld.rng, false, true, worldNormal, texAlbedo)) { do_skip(); return; }
        pld.color = texAlbedo;
        pld.albedo = pld.color;
        pld.emission = load3<T>(m.emission);
        pld.rayOrigin = offsetAlongNormal(hit.worldPosition, hit.worldNormalGeometry);
        pld.rayDirection = fuzzyReflection<T>(dir, worldNormal, (T)m.roughness, pld.rng);
        pld.rayHitSky = false;
        pld.skip = false;
        pld.insideDielectric = false;
        pld.materialID = 1;
        pld.surfaceNormal = worldNormal;
        pld.pdf = 0;
        pld.tbn = hit.tbn;
        pld.props = &m;
        pld.didRefract = false;
        pld.eta = 0;
        pld.accumulatedDistance = 0;
    } else if (m.material_idx == 2) {   // dielectric.rchit.glsl:40-113
        const T ior = (T)m.ior;
        const T ri = hit.frontFace ? (T)1 / ior : ior;
        const Vec3<T> unitDir = normalize(dir);
        const T cosT = std::min(dot(-unitDir, hit.worldNormal), (T)1);
        const T sinT = std::sqrt((T)1 - cosT * cosT);
        const bool cannot = ri * sinT > (T)1;
        const T refl = reflectance(cosT, ri);
        const bool prevInside = pld.insideDielectric;
        apply_textures(c.s, hit, m, dir, pld.rng, false, false, worldNormal, texAlbedo);
        const Vec3<T> albedo = texAlbedo;
        if (cannot || refl > rng_random<T>(pld.rng)) {
            pld.rayDirection = fuzzyReflection<T>(unitDir, worldNormal, (T)m.roughness, pld.rng);
            pld.color = Vec3<T>((T)1, (T)1, (T)1);
            pld.rayOrigin = offsetAlongNormal(hit.worldPosition, hit.worldNormalGeometry);
        } else {
            pld.insideDielectric = hit.frontFace;
            pld.rayDirection = refract(unitDir, worldNormal, ri) + randomUnitVec<T>(pld.rng) * (T)m.roughness;
            pld.color = albedo;
            pld.rayOrigin = offsetForDielectric(hit.worldPosition, hit.worldNormalGeometry, unitDir);
        }
        pld.accumulatedDistance += prevInside ? length(hit.worldPosition - org) : (T)0;
        if (prevInside && !pld.insideDielectric) {
            pld.color = Vec3<T>((T)1, (T)1, (T)1) * std::exp(-(T)m.absorption * pld.accumulatedDistance);
            pld.color = pld.color * albedo;
            pld.accumulatedDistance = 0;
        }
        pld.albedo = pld.color;
        pld.emission = load3<T>(m.emission);
        pld.rayHitSky = false;
        pld.skip = false;
        pld.materialID = 2;
        pld.surfaceNormal = worldNormal;
        pld.pdf = 0;
        pld.tbn = hit.tbn;
        pld.props = &m;
        pld.didRefract = false;
        pld.eta = 0;
    } else {   // disney.rchit.glsl:36-198
        if (m.cull_backface && !hit.frontFace) { do_skip(); return; }
        if (!apply_textures(c.s, hit, m, dir, pld.rng, true, true, worldNormal, texAlbedo)) { do_skip(); return; }
        const Vec3<T> albedo = texAlbedo;
        const T ior = (T)m.ior;
        const T eta = hit.frontFace ? (T)1 / ior : ior;
        const DisneyParams<T> p = disney_params<T>(m, albedo);
        bool didRefract = false, choseGlass = false;
        const Vec3<T> wi = -dir;
        const Vec3<T> rayDir = sampleDisney(hit.tbn, p, eta, worldNormal, wi, didRefract, choseGlass, pld.rng);
        const Vec3<T> h = normalize(rayDir + wi);
        T pdf;
        const Vec3<T> f = evalDisney(hit.tbn, p, eta, didRefract, worldNormal, wi, rayDir, h, pdf);
        const T cosI = std::max(dot(worldNormal, rayDir), (T)0);
        pld.color = f * cosI / pdf;
        pld.albedo = albedo;
        pld.pdf = pdf;
        pld.emission = load3<T>(m.emission);
        pld.rayOrigin = offsetForDielectric(hit.worldPosition, hit.worldNormalGeometry, rayDir);
        pld.rayDirection = rayDir;
        pld.rayHitSky = false;
        pld.skip = false;
        pld.materialID = 3;
        pld.surfaceNormal = worldNormal;
        pld.tbn = hit.tbn;
        pld.props = &m;
        pld.didRefract = false;
        pld.eta = 0;
        pld.insideDielectric = choseGlass;
        if (pld.insideDielectric) pld.accumulatedDistance += length(hit.worldPosition - org);
        else pld.accumulatedDistance = 0;
    }
}

// nee.h.glsl:52-124 randomEmissivePoint, with indices past the end of the model (possible when the
// triangle CDF index of a non-first emissive instance is used as a model-relative index) returning no
// sample (valid = false) instead of reading out of range.
template <class T>
struct LightSample {
    Vec3<T> point, normal, emission;
    T pdf = 0;
    bool cull = false, valid = false;
};

template <class T>
LightSample<T> randomEmissivePoint(const Ctx<T>& c, uint32_t& rng) {
    const OScene& s = c.s;
    LightSample<T> ls;
    const T u0 = rng_random<T>(rng);
    int lo = 0, hi = (int)s.emissive.size() - 1;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (u0 <= (T)s.cdf_instances[mid]) hi = mid;
        else lo = mid + 1;
    }
    const uint32_t ie = (uint32_t)lo;
    const OInstance& inst = s.instances[s.emissive[ie]];
    const T u1 = rng_random<T>(rng);
    lo = (int)inst.cdf_start;
    hi = (int)inst.cdf_end;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (u1 <= (T)s.cdf_triangles[mid]) hi = mid;
        else lo = mid + 1;
    }
    const uint32_t tri = (uint32_t)lo;
    const OObject& o = s.objects[inst.obj];
    // consume the two draws of randomPointOnTriangle even when the sample is invalid
    const T r1 = rng_random<T>(rng), r2 = rng_random<T>(rng);
    if (3ull * tri + 2 >= o.idx.size()) return ls;
    Vec3<T> v0 = load3<T>(&o.v[4 * o.idx[3 * tri]]), v1 = load3<T>(&o.v[4 * o.idx[3 * tri + 1]]),
            v2 = load3<T>(&o.v[4 * o.idx[3 * tri + 2]]);
    v0 = xform_point(inst.T, v0);
    v1 = xform_point(inst.T, v1);
    v2 = xform_point(inst.T, v2);
    const T beta = (T)1 - std::sqrt(r1);
    const T gamma = ((T)1 - beta) * r2;
    const T alpha = (T)1 - beta - gamma;
    ls.point = v0 * alpha + v1 * beta + v2 * gamma;
    ls.normal = normalize(cross(v1 - v0, v2 - v0));
    ls.emission = load3<T>(inst.mats[0].emission);
    ls.pdf = ((T)inst.weight / (T)c.pc.totalEmissiveWeight) * ((T)1 / (T)inst.area);
    ls.cull = inst.mats[0].cull_backface != 0;
    ls.valid = true;
    return ls;
}

// raytrace.rgen.glsl:43-95 directLight; returns (light, pdf) and the BSDF pdf of the light direction.
template <class T>
void directLight(const Ctx<T>& c, const Payload<T>& pld, Vec3<T> rayIn, uint32_t& rng, Vec3<T>& light, T& pdf_light,
                 T& pdf_bsdf) {
    light = Vec3<T>((T)0, (T)0, (T)0);
    pdf_light = 0;
    pdf_bsdf = 0;
    const LightSample<T> t = randomEmissivePoint(c, rng);
    if (!t.valid) return;
    const Vec3<T> dvec = t.point - pld.rayOrigin;
    const Vec3<T> direction = normalize(dvec);
    const T dist = length(dvec);
    pdf_light = t.pdf * dist * dist / std::max(dot(t.normal, -direction), (T)0.0001);
    Vec3<T> brdf;
    if (pld.materialID == 0) {
        brdf = pld.albedo / kpi<T>();
        pdf_bsdf = pdfLambertian(pld.surfaceNormal, direction);
    } else {
        const Vec3<T> h = normalize(direction + -rayIn);
        const DisneyParams<T> p = disney_params<T>(*pld.props, pld.albedo);
        brdf = evalDisney(pld.tbn, p, pld.eta, pld.didRefract, pld.surfaceNormal, -rayIn, direction, h, pdf_bsdf);
    }
    RayRec sr{(float)pld.rayOrigin.x, (float)pld.rayOrigin.y, (float)pld.rayOrigin.z, 0.0f,
              (float)direction.x, (float)direction.y, (float)direction.z, (float)(dist - (T)0.001)};
    if (trace_occluded(c.s.bvh, sr, c.precision)) return;
    T cosI = dot(pld.surfaceNormal, direction);
    cosI = t.cull ? std::max(cosI, (T)0) : std::fabs(cosI);
    T gnum = dot(t.normal, -direction);
    gnum = t.cull ? std::max(gnum, (T)0) : std::fabs(gnum);
    const T G = gnum / (dist * dist);
    light = t.emission * brdf * (cosI * G / t.pdf);
}

// Light pdf (solid angle) of reaching `p` on the emissive triangle `prim` from `from` (emission MIS).
template <class T>
T light_pdf_sa(const Ctx<T>& c, uint32_t prim, Vec3<T> from, Vec3<T> p) {
    const OInstance& inst = c.s.instances[c.s.prim_inst[prim]];
    if (!inst.emissive) return 0;
    const OObject& o = c.s.objects[inst.obj];
    const uint32_t lp = prim - inst.first_prim;
    const Vec3<T> v0 = xform_point(inst.T, load3<T>(&o.v[4 * o.idx[3 * lp]]));
    const Vec3<T> v1 = xform_point(inst.T, load3<T>(&o.v[4 * o.idx[3 * lp + 1]]));
    const Vec3<T> v2 = xform_point(inst.T, load3<T>(&o.v[4 * o.idx[3 * lp + 2]]));
    const Vec3<T> n = normalize(cross(v1 - v0, v2 - v0));
    const Vec3<T> dvec = p - from;
    const T dist = length(dvec);
    const Vec3<T> dir = dvec / dist;
    const T pdf_area = ((T)inst.weight / (T)c.pc.totalEmissiveWeight) * ((T)1 / (T)inst.area);
    return pdf_area * dist * dist / std::max(dot(n, -dir), (T)0.0001);
}

inline uint32_t seed_hash(uint32_t pixel, uint32_t sample, uint32_t seed) {
    // Per-path seed for the nee_mis mode: a murmur3-style finalizer over the three keys.
    uint32_t h = seed * 0x9E3779B1u ^ (pixel * 0x85EBCA77u + 0x165667B1u) ^ (sample * 0xC2B2AE3Du + 0x27D4EB2Fu);
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}

template <class T>
struct SegResult {
    Vec3<T> radiance;
};

// raytrace.rgen.glsl:97-184 traceSegments; accumulatedDistance lives in `accDist` across samples.
template <class T>
Vec3<T> traceSegments(const Ctx<T>& c, Vec3<T> org, Vec3<T> dir, uint32_t& rng, T& accDist) {
    Payload<T> pld;
    pld.rng = rng;
    pld.accumulatedDistance = accDist;
    pld.insideDielectric = false;
    Vec3<T> thr((T)1, (T)1, (T)1), inc((T)0, (T)0, (T)0);
    const bool nee = c.opt.mode == 1;
    bool prevNEE = false;     // nee_mis: whether the previous processed vertex sampled a light
    T prevPdf = 0;            // nee_mis: BSDF pdf of the direction sampled at that vertex
    for (uint32_t seg = 0; seg < c.pc.maxBounces; ++seg) {
        const Vec3<T> rayIn = dir;
        const Vec3<T> rayOrg = org;
        trace_and_shade(c, org, dir, pld);
        org = pld.rayOrigin;
        dir = pld.rayDirection;
        if (pld.skip) {
            prevNEE = false;
            continue;
        }
        if (pld.rayHitSky) {
            inc = inc + pld.color * thr;
            break;
        }
        if (!pld.insideDielectric) {
            Vec3<T> contrib = pld.emission;
            if (nee) {
                T wb = 1;
                if (prevNEE && (pld.emission.x != 0 || pld.emission.y != 0 || pld.emission.z != 0)) {
                    const T hitT = 0;
                    (void)hitT;
                    // hit point of this segment: reconstruct from the payload's surface (the origin of
                    // the next ray is offset by a few ulps; use the light pdf at the offset origin).
                    const T pl = light_pdf_sa(c, pld.prim, rayOrg, pld.rayOrigin);
                    wb = powerHeuristic(prevPdf, pl);
                }
                contrib = contrib * wb;
                const bool doNEE = pld.materialID == 0 || pld.materialID == 3;
                if (doNEE && !c.s.emissive.empty()) {
                    Vec3<T> L;
                    T pl, pb;
                    directLight(c, pld, rayIn, pld.rng, L, pl, pb);
                    if (pl > 0) contrib = contrib + L * powerHeuristic(pl, pb);
                }
                prevNEE = doNEE && !c.s.emissive.empty();
                prevPdf = pld.pdf;
            }
            inc = inc + contrib * thr;
            thr = thr * pld.color;
        } else {
            prevNEE = false;
        }
    }
    rng = pld.rng;
    accDist = pld.accumulatedDistance;
    return inc;
}

// raytrace.rgen.glsl:34-41, 194-247
template <class T>
void getStartingRay(const Ctx<T>& c, uint32_t px, uint32_t py, uint32_t W, uint32_t H, uint32_t& rng, Vec3<T>& org,
                    Vec3<T>& dir) {
    const T u1 = std::max((T)1e-5, rng_random<T>(rng));
    const T u2 = rng_random<T>(rng);
    const T r = std::sqrt((T)-2 * std::log(u1));
    const T theta = (T)2 * kpi<T>() * u2;
    const T gx = r * std::cos(theta), gy = r * std::sin(theta);
    const T cx = (T)px + (T)0.5 + (T)0.375 * gx;
    const T cy = (T)py + (T)0.5 + (T)0.375 * gy;
    const T ndcx = (cx / (T)W) * (T)2 - (T)1;
    const T ndcy = -((cy / (T)H) * (T)2 - (T)1);
    const float* P = c.pc.invProjection;
    T vp[4];
    const T clip[4] = {ndcx, ndcy, (T)-1, (T)1};
    for (int k = 0; k < 4; ++k)
        vp[k] = (T)P[0 * 4 + k] * clip[0] + (T)P[1 * 4 + k] * clip[1] + (T)P[2 * 4 + k] * clip[2] + (T)P[3 * 4 + k] * clip[3];
    for (int k = 0; k < 4; ++k) vp[k] = vp[k] / vp[3];
    const Vec3<T> viewDir = normalize(Vec3<T>(vp[0], vp[1], vp[2]));
    const float* V = c.pc.invView;
    Vec3<T> wd;
    for (int k = 0; k < 3; ++k) wd[k] = (T)V[0 * 4 + k] * viewDir.x + (T)V[1 * 4 + k] * viewDir.y + (T)V[2 * 4 + k] * viewDir.z;
    const Vec3<T> rd = normalize(wd);
    const Vec3<T> origin = load3<T>(V + 12);
    const Vec3<T> focal = origin + rd * (T)c.pc.focusDist;
    // randomInUnitHexagon receives the state by value: its draws do not advance the path's RNG.
    uint32_t hs = rng;
    T hx, hy;
    const T sqrt3 = (T)1.73205080757;
    do {
        hx = (T)2 * rng_random<T>(hs) - (T)1;
        hy = (rng_random<T>(hs) - (T)0.5) * sqrt3;
    } while (std::fabs(hy) > sqrt3 * (T)0.5 || (sqrt3 * std::fabs(hx) + std::fabs(hy)) > sqrt3);
    const T lx = hx * (T)c.pc.defocusMultiplier, ly = hy * (T)c.pc.defocusMultiplier;
    const Vec3<T> right = normalize(load3<T>(V + 0));
    const Vec3<T> up = normalize(load3<T>(V + 4));
    org = origin + right * lx + up * ly;
    dir = normalize(focal - org);
}

template <class T>
void render_pixel(const Ctx<T>& c, uint32_t x, uint32_t y, uint32_t W, uint32_t H, float* accum, float* samples) {
    const uint32_t spp = c.pc.samplesPerPixel;
    const uint32_t pixel = y * W + x;
    uint32_t rng = (c.pc.sampleBatch * H + y) * W + x;
    T accDist = 0;
    int actual = 0;
    Vec3<T> sum((T)0, (T)0, (T)0);
    for (uint32_t s = 0; s < spp; ++s) {
        if (c.opt.mode == 1) {
            rng = seed_hash(pixel, c.pc.sampleBatch * spp + s, c.opt.seed);
            accDist = 0;
        }
        Vec3<T> org, dir;
        getStartingRay(c, x, y, W, H, rng, org, dir);
        Vec3<T> col = traceSegments(c, org, dir, rng, accDist);
        // clamp keeps NaN (the NaN test below is how the reference drops such samples)
        for (int k = 0; k < 3; ++k)
            if (!std::isnan(col[k])) col[k] = clampT(col[k], (T)0, (T)c.pc.directClamp);
        if (samples) {
            float* o = samples + 3ull * ((uint64_t)pixel * spp + s);
            o[0] = (float)col.x; o[1] = (float)col.y; o[2] = (float)col.z;
        }
        if (std::isnan(col.x) || std::isnan(col.y) || std::isnan(col.z)) continue;
        actual++;
        sum = sum + col;
    }
    Vec3<T> fin = sum / (T)actual;
    float* a = accum + 4ull * pixel;
    if (c.pc.sampleBatch > 0) {
        const Vec3<T> prev((T)a[0], (T)a[1], (T)a[2]);
        fin = (prev * (T)c.pc.sampleBatch + fin) / (T)(c.pc.sampleBatch + 1);
    }
    a[0] = (float)fin.x; a[1] = (float)fin.y; a[2] = (float)fin.z; a[3] = 1.0f;
}

void finalize_scene(OScene& s) {
    uint64_t total = 0;
    for (OInstance& inst : s.instances) {
        inst.first_prim = (uint32_t)total;
        total += s.objects[inst.obj].idx.size() / 3;
    }
    s.world.resize(9 * total);
    s.prim_inst.resize(total);
    for (size_t ii = 0; ii < s.instances.size(); ++ii) {
        OInstance& inst = s.instances[ii];
        const OObject& o = s.objects[inst.obj];
        const size_t nt = o.idx.size() / 3;
        for (size_t t = 0; t < nt; ++t) {
            const uint64_t g = inst.first_prim + t;
            s.prim_inst[g] = (uint32_t)ii;
            for (int j = 0; j < 3; ++j) {
                const float* v = &o.v[4 * o.idx[3 * t + j]];
                for (int r = 0; r < 3; ++r) {
                    float acc = inst.T[0 * 4 + r] * v[0];
                    acc = acc + inst.T[1 * 4 + r] * v[1];
                    acc = acc + inst.T[2 * 4 + r] * v[2];
                    acc = acc + inst.T[3 * 4 + r];
                    s.world[9 * g + 3 * j + r] = acc;
                }
            }
        }
        // Instance::computeCDF (src/scene/Instance.cpp:15-53) for single-material emissive instances
        inst.emissive = false;
        if (!inst.face_mat.empty()) continue;
        const float* e = inst.mats[0].emission;
        if (!(e[0] * e[0] + e[1] * e[1] + e[2] * e[2] > 0.00001f * 0.00001f)) continue;
        inst.emissive = true;
        const float bright = (float)(0.2126 * e[0] + 0.7152 * e[1] + 0.0722 * e[2]);
        const size_t nv = o.v.size() / 4;
        std::vector<float> tv(3 * nv);
        for (size_t i = 0; i < nv; ++i)
            for (int cc = 0; cc < 3; ++cc) {   // row vector times matrix: the transpose of M applied
                const float* col = inst.T + 4 * cc;
                float acc = col[0] * o.v[4 * i];
                acc = acc + col[1] * o.v[4 * i + 1];
                acc = acc + col[2] * o.v[4 * i + 2];
                acc = acc + col[3] * 1.0f;
                tv[3 * i + cc] = acc;
            }
        inst.cdf.resize(nt);
        float cum = 0, area = 0;
        for (size_t t = 0; t < nt; ++t) {
            const float* a = &tv[3 * o.idx[3 * t]];
            const float* b = &tv[3 * o.idx[3 * t + 1]];
            const float* cpt = &tv[3 * o.idx[3 * t + 2]];
            const float ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
            const float ac[3] = {cpt[0] - a[0], cpt[1] - a[1], cpt[2] - a[2]};
            const float cr[3] = {ab[1] * ac[2] - ac[1] * ab[2], ab[2] * ac[0] - ac[2] * ab[0], ab[0] * ac[1] - ac[0] * ab[1]};
            const float ta = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]) / 2.0f;
            area += ta;
            cum += ta * bright;
            inst.cdf[t] = cum;
        }
        for (float& v : inst.cdf) v /= cum;
        inst.weight = cum;
        inst.area = area;
    }
    // Instances::computeSamplingDataEmissives (src/scene/Instances.cpp:52-114), without the CDF
    // deduplication (duplicates share identical CDF contents, so sampling is unchanged).
    s.emissive.clear();
    s.cdf_triangles.clear();
    for (size_t ii = 0; ii < s.instances.size(); ++ii) {
        OInstance& inst = s.instances[ii];
        if (!inst.emissive) continue;
        s.emissive.push_back((uint32_t)ii);
        inst.cdf_start = (uint32_t)s.cdf_triangles.size();
        inst.cdf_end = inst.cdf_start + (uint32_t)inst.cdf.size() - 1;
        s.cdf_triangles.insert(s.cdf_triangles.end(), inst.cdf.begin(), inst.cdf.end());
    }
    s.cdf_instances.assign(s.emissive.size(), 0.0f);
    float cum = 0;
    for (size_t i = 0; i < s.emissive.size(); ++i) {
        cum += s.instances[s.emissive[i]].weight;
        s.cdf_instances[i] = cum;
    }
    for (float& v : s.cdf_instances) v /= cum;
    s.total_weight = cum;
    if (s.bvh) oracle_bvh_destroy(s.bvh);
    s.bvh = oracle_bvh_build(s.world.data(), total);
}

}  // namespace oracle

using namespace oracle;

extern "C" {

void* oracle_scene_new(void) { return new OScene(); }

void oracle_scene_free(void* h) {
    OScene* s = static_cast<OScene*>(h);
    if (!s) return;
    if (s->bvh) oracle_bvh_destroy(s->bvh);
    delete s;
}

uint32_t oracle_scene_add_object(void* h, const float* v4, uint64_t nv, const uint32_t* idx, uint64_t nidx,
                                 const float* tbn9, uint64_t ntbn, const uint32_t* tbn_idx, uint64_t ntbn_idx,
                                 const float* uv2, uint64_t nuv, const uint32_t* uv_idx, uint64_t nuv_idx) {
    OScene* s = static_cast<OScene*>(h);
    OObject o;
    o.v.assign(v4, v4 + 4 * nv);
    o.idx.assign(idx, idx + nidx);
    if (tbn9 && ntbn) o.tbn.assign(tbn9, tbn9 + 9 * ntbn);
    if (tbn_idx && ntbn_idx) o.tbn_idx.assign(tbn_idx, tbn_idx + ntbn_idx);
    if (uv2 && nuv) o.uv.assign(uv2, uv2 + 2 * nuv);
    if (uv_idx && nuv_idx) o.uv_idx.assign(uv_idx, uv_idx + nuv_idx);
    s->objects.push_back(std::move(o));
    return (uint32_t)(s->objects.size() - 1);
}

void oracle_scene_add_instance(void* h, uint32_t obj, const float* T16, const OMaterial* mats, uint32_t nmat,
                               const uint32_t* face_mat) {
    OScene* s = static_cast<OScene*>(h);
    OInstance inst;
    inst.obj = obj;
    std::memcpy(inst.T, T16, sizeof(inst.T));
    inst.mats.assign(mats, mats + nmat);
    if (face_mat) inst.face_mat.assign(face_mat, face_mat + s->objects[obj].idx.size() / 3);
    s->instances.push_back(std::move(inst));
}

uint32_t oracle_scene_add_texture(void* h, const uint8_t* rgba8, uint32_t w, uint32_t hgt) {
    OScene* s = static_cast<OScene*>(h);
    OTexture t;
    t.w = w;
    t.h = hgt;
    t.texels.resize((size_t)w * hgt);
    for (size_t i = 0; i < t.texels.size(); ++i)
        t.texels[i] = (uint32_t)rgba8[4 * i] | ((uint32_t)rgba8[4 * i + 1] << 8) | ((uint32_t)rgba8[4 * i + 2] << 16) |
                      ((uint32_t)rgba8[4 * i + 3] << 24);
    s->textures.push_back(std::move(t));
    return (uint32_t)(s->textures.size() - 1);
}

void oracle_scene_finalize(void* h) { finalize_scene(*static_cast<OScene*>(h)); }

float oracle_scene_emissive_weight(void* h) { return static_cast<OScene*>(h)->total_weight; }

// Renders the window [x0, x1) x [y0, y1) of a W x H frame into accum (W*H*4 floats, read for the
// running mean when sampleBatch > 0) and optionally the per-sample colours (W*H*spp*3 floats).
void oracle_render(void* h, const OPush* pc, const ORenderOptions* opt, uint32_t W, uint32_t H, int precision,
                   int threads, float* accum, float* samples) {
    const OScene& s = *static_cast<OScene*>(h);
    const uint32_t x0 = opt->x0, y0 = opt->y0, x1 = std::min(opt->x1, W), y1 = std::min(opt->y1, H);
    const uint64_t n = (uint64_t)(x1 - x0) * (y1 - y0);
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint64_t> next{0};
    auto work = [&] {
        for (;;) {
            const uint64_t b = next.fetch_add(16);
            if (b >= n) break;
            for (uint64_t i = b; i < std::min(n, b + 16); ++i) {
                const uint32_t x = x0 + (uint32_t)(i % (x1 - x0)), y = y0 + (uint32_t)(i / (x1 - x0));
                if (precision == 64) render_pixel<double>(Ctx<double>{s, *pc, *opt, 64}, x, y, W, H, accum, samples);
                else render_pixel<float>(Ctx<float>{s, *pc, *opt, 32}, x, y, W, H, accum, samples);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}

uint32_t oracle_seed_hash(uint32_t pixel, uint32_t sample, uint32_t seed) { return seed_hash(pixel, sample, seed); }

}  // extern "C"
