// ORACLE — test infrastructure only (see oracle_common.h).
//
// Known-answer entry points for single shading functions, evaluated on 40-float case records (the same
// layout the library's device self-check reads):
//   kind 0  offsetPositionAlongNormal (closestHitCommon.h.glsl:156-177): p = r[0..2], n = r[3..5] -> 3
//   kind 1  sampleGGXVNDF (brdfDisney.h.glsl:9-40): V = r[0..2], ax = r[6], ay = r[7], RNG state =
//           bits of r[8] -> the half vector (3) and the RNG state after its two draws (bits, 4th output)
//   kind 2  evalDisney (brdfDisney.h.glsl:656-711): base r[0..2], specTint r[3..5], sheenTint r[6..8],
//           anisotropic r[9], roughness r[10], subsurface r[11], clearcoatGloss r[12], metallic r[13],
//           clearcoat r[14], specularTransmission r[15], sheen r[16], eta r[17], didRefract r[18] != 0,
//           n r[19..21], wi r[22..24], wo r[25..27], TBN columns r[28..36]; h = normalize(wo + wi)
//           -> f (3) and pdf
//   kind 3  random (shaderCommon.h.glsl:39-45): state = bits of r[0] -> six draws, the state after (o6)
//   kind 4  offsetPositionForDielectric (dielectric.rchit.glsl:14-38): p r[0..2], n r[3..5], dir r[6..8] -> 3
//   kind 5  sampleDisney (brdfDisney.h.glsl:609-654): TBN r[28..36], base r[0..2], anisotropic r[9],
//           roughness r[10], clearcoatGloss r[12], eta r[17], metallic r[13], clearcoat r[14],
//           specularTransmission r[15], n r[19..21], wi r[22..24], state = bits of r[37]
//           -> the direction (3), didRefract, choseGlass, the state after
//   kind 6  diffuseReflection (closestHitCommon.h.glsl:215-222): n r[0..2], state bits r[8] -> 3, state
//   kind 7  randomUnitVec (closestHitCommon.h.glsl:195-205): state bits r[8] -> 3, state
//   kind 10 reflectance (dielectric.rchit.glsl:7-12; the same expression as brdfDisney.h.glsl:389-394):
//           cos r[0], ri r[1] -> o0
//   kind 14 pdfMetal, pdfClearcoat (o0, o1; o2 unused), pdfLambertian(n, wo) (o3), the power heuristic of
//           pdf.h.glsl:4-7 on r[38], r[39] (o4), luminance(base) (o5)
// oracle_kat8 writes 8 doubles per case; oracle_kat the first 4 (the float result widened in precision 32).
#include <cstdint>
#include <cstring>

#include "oracle_bsdf.h"
#include "oracle_common.h"

namespace {

using namespace oracle;

template <class T>
DisneyParams<T> disney_params(const float* r) {
    auto v3 = [&](int i) { return Vec3<T>((T)r[i], (T)r[i + 1], (T)r[i + 2]); };
    DisneyParams<T> p;
    p.base = v3(0);
    p.specTint = v3(3);
    p.sheenTint = v3(6);
    p.aniso = (T)r[9]; p.rough = (T)r[10]; p.subsurface = (T)r[11]; p.ccGloss = (T)r[12];
    p.metallic = (T)r[13]; p.clearcoat = (T)r[14]; p.specTrans = (T)r[15]; p.sheen = (T)r[16];
    return p;
}

template <class T>
void eval_case(int kind, const float* r, double* o) {
    auto v3 = [&](int i) { return Vec3<T>((T)r[i], (T)r[i + 1], (T)r[i + 2]); };
    auto bits = [&](int i) { uint32_t s; std::memcpy(&s, r + i, 4); return s; };
    for (int k = 0; k < 8; ++k) o[k] = 0.0;
    const Mat3<T> frame{v3(28), v3(31), v3(34)};
    if (kind == 3) {
        uint32_t s = bits(0);
        for (int k = 0; k < 6; ++k) o[k] = (double)rng_random<T>(s);
        o[6] = (double)s;
        return;
    }
    if (kind == 4) {
        const Vec3<T> q = offsetForDielectric(v3(0), v3(3), v3(6));
        o[0] = (double)q.x; o[1] = (double)q.y; o[2] = (double)q.z;
        return;
    }
    if (kind == 5) {
        uint32_t s = bits(37);
        bool refr = false, glass = false;
        const Vec3<T> wo = sampleDisney(frame, disney_params<T>(r), (T)r[17], v3(19), v3(22), refr, glass, s);
        o[0] = (double)wo.x; o[1] = (double)wo.y; o[2] = (double)wo.z; o[3] = refr; o[4] = glass; o[5] = (double)s;
        return;
    }
    if (kind == 6 || kind == 7) {
        uint32_t s = bits(8);
        const Vec3<T> d = kind == 6 ? diffuseReflection(v3(0), s) : randomUnitVec<T>(s);
        o[0] = (double)d.x; o[1] = (double)d.y; o[2] = (double)d.z; o[3] = (double)s;
        return;
    }
    if (kind == 10) {
        o[0] = (double)reflectance((T)r[0], (T)r[1]);
        return;
    }
    if (kind == 14) {
        const Vec3<T> wi = v3(22), wo = v3(25);
        const Vec3<T> h = normalize(wo + wi);
        o[0] = (double)pdfMetal(frame, wi, wo, (T)r[9], (T)r[10]);
        o[1] = (double)pdfClearcoat(frame, wi, wo, h, (T)r[12]);
        o[3] = (double)pdfLambertian(v3(19), wo);
        o[4] = (double)powerHeuristic((T)r[38], (T)r[39]);
        o[5] = (double)luminance(v3(0));
        return;
    }
    if (kind == 0) {
        const Vec3<T> q = offsetAlongNormal(v3(0), v3(3));
        o[0] = (double)q.x; o[1] = (double)q.y; o[2] = (double)q.z;
    } else if (kind == 1) {
        uint32_t s;
        std::memcpy(&s, r + 8, 4);
        const Vec3<T> h = sampleGGXVNDF(v3(0), (T)r[6], (T)r[7], s);
        o[0] = (double)h.x; o[1] = (double)h.y; o[2] = (double)h.z; o[3] = (double)s;
    } else {
        DisneyParams<T> p;
        p.base = v3(0);
        p.specTint = v3(3);
        p.sheenTint = v3(6);
        p.aniso = (T)r[9]; p.rough = (T)r[10]; p.subsurface = (T)r[11]; p.ccGloss = (T)r[12];
        p.metallic = (T)r[13]; p.clearcoat = (T)r[14]; p.specTrans = (T)r[15]; p.sheen = (T)r[16];
        const Mat3<T> tbn{v3(28), v3(31), v3(34)};
        const Vec3<T> wi = v3(22), wo = v3(25);
        const Vec3<T> h = normalize(wo + wi);
        T pdf;
        const Vec3<T> f = evalDisney(tbn, p, (T)r[17], r[18] != 0.0f, v3(19), wi, wo, h, pdf);
        o[0] = (double)f.x; o[1] = (double)f.y; o[2] = (double)f.z; o[3] = (double)pdf;
    }
}

}  // namespace

extern "C" void oracle_kat8(int kind, const float* records, uint64_t n, int precision, double* out) {
    for (uint64_t i = 0; i < n; ++i) {
        if (precision == 64) eval_case<double>(kind, records + 40 * i, out + 8 * i);
        else eval_case<float>(kind, records + 40 * i, out + 8 * i);
    }
}

extern "C" void oracle_kat(int kind, const float* records, uint64_t n, int precision, double* out) {
    for (uint64_t i = 0; i < n; ++i) {
        double o8[8];
        oracle_kat8(kind, records + 40 * i, 1, precision, o8);
        std::memcpy(out + 4 * i, o8, 4 * sizeof(double));
    }
}
