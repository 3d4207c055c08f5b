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
// Outputs are 4 doubles per case (the float result widened in precision 32).
#include <cstdint>
#include <cstring>

#include "oracle_bsdf.h"
#include "oracle_common.h"

namespace {

using namespace oracle;

template <class T>
void eval_case(int kind, const float* r, double* o) {
    auto v3 = [&](int i) { return Vec3<T>((T)r[i], (T)r[i + 1], (T)r[i + 2]); };
    o[0] = o[1] = o[2] = o[3] = 0.0;
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

extern "C" void oracle_kat(int kind, const float* records, uint64_t n, int precision, double* out) {
    for (uint64_t i = 0; i < n; ++i) {
        if (precision == 64) eval_case<double>(kind, records + 40 * i, out + 4 * i);
        else eval_case<float>(kind, records + 40 * i, out + 4 * i);
    }
}
