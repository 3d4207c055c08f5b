// Device self-check of single shading functions on fixed inputs (the device code the integrators run,
// evaluated one case per thread).  Case records hold 40 floats:
//   kind 0  offset_along_normal (closestHitCommon.h.glsl:156-177): p = r[0..2], n = r[3..5] -> 3 floats
//   kind 1  sample_ggx_vndf (brdfDisney.h.glsl:9-40): V = r[0..2], ax = r[6], ay = r[7], RNG state = bits
//           of r[8] -> the half vector and, as the 4th output's bits, the RNG state after its two draws
//   kind 2  eval_disney (brdfDisney.h.glsl:656-711): base r[0..2], specTint r[3..5], sheenTint r[6..8],
//           anisotropic r[9], roughness r[10], subsurface r[11], clearcoatGloss r[12], metallic r[13],
//           clearcoat r[14], specularTransmission r[15], sheen r[16], eta r[17], didRefract r[18] != 0,
//           n r[19..21], wi r[22..24], wo r[25..27], TBN columns r[28..36]; h = normalize(wo + wi)
//           -> f (3 floats) and the pdf
//   kind 3  rng_next (shaderCommon.h.glsl:39-45): state = bits of r[0] -> three draws, the state after
//           (bits, 4th output)
//   kind 4  offset_for_dielectric (dielectric.rchit.glsl:14-38): p = r[0..2], n = r[3..5], dir = r[6..8]
//   kind 5  sample_disney (brdfDisney.h.glsl:609-654): TBN r[28..36], base r[0..2], anisotropic r[9],
//           roughness r[10], clearcoatGloss r[12], eta r[17], metallic r[13], clearcoat r[14],
//           specularTransmission r[15], n r[19..21], wi r[22..24], state = bits of r[37] -> the sampled
//           direction and the state after (bits)
//   kind 15 the same sample -> didRefract, choseGlass (0 or 1)
//   kind 6  diffuse_reflection (closestHitCommon.h.glsl:215-222): n = r[0..2], state = bits of r[8]
//           -> the direction and the state after (bits)
//   kind 7  random_unit_vec (closestHitCommon.h.glsl:195-205): state = bits of r[8] -> 3, state after
#include "kat.h"

#include "shading_device.cuh"

namespace rt {

__global__ void k_kat(int kind, const float* __restrict__ rec, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rec + 40ull * i;
    float* o = out + 4ull * i;
    auto v3 = [&](int k) { return V3{r[k], r[k + 1], r[k + 2]}; };
    o[0] = o[1] = o[2] = o[3] = 0.0f;
    if (kind == 0) {
        const V3 q = offset_along_normal(v3(0), v3(3));
        o[0] = q.x; o[1] = q.y; o[2] = q.z;
    } else if (kind == 1) {
        uint32_t s = __float_as_uint(r[8]);
        const V3 h = sample_ggx_vndf(v3(0), r[6], r[7], s);
        o[0] = h.x; o[1] = h.y; o[2] = h.z;
        o[3] = __uint_as_float(s);
    } else if (kind == 3) {
        uint32_t s = __float_as_uint(r[0]);
        o[0] = rng_next(s); o[1] = rng_next(s); o[2] = rng_next(s);
        o[3] = __uint_as_float(s);
    } else if (kind == 4) {
        const V3 q = offset_for_dielectric(v3(0), v3(3), v3(6));
        o[0] = q.x; o[1] = q.y; o[2] = q.z;
    } else if (kind == 5 || kind == 15) {
        DisneyParams p;
        p.base = v3(0);
        p.specTint = V3{1.0f, 1.0f, 1.0f};
        p.sheenTint = V3{1.0f, 1.0f, 1.0f};
        p.aniso = r[9]; p.rough = r[10]; p.subsurface = 0.0f; p.ccGloss = r[12];
        p.metallic = r[13]; p.clearcoat = r[14]; p.specTrans = r[15]; p.sheen = 0.0f;
        const M3 tbn{v3(28), v3(31), v3(34)};
        uint32_t s = __float_as_uint(r[37]);
        bool refracted = false, glass = false;
        const V3 wo = sample_disney(tbn, p, r[17], v3(19), v3(22), refracted, glass, s);
        if (kind == 5) {
            o[0] = wo.x; o[1] = wo.y; o[2] = wo.z; o[3] = __uint_as_float(s);
        } else {
            o[0] = refracted ? 1.0f : 0.0f; o[1] = glass ? 1.0f : 0.0f;
        }
    } else if (kind == 6 || kind == 7) {
        uint32_t s = __float_as_uint(r[8]);
        const V3 d = kind == 6 ? diffuse_reflection(v3(0), s) : random_unit_vec(s);
        o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = __uint_as_float(s);
    } else {
        DisneyParams p;
        p.base = v3(0);
        p.specTint = v3(3);
        p.sheenTint = v3(6);
        p.aniso = r[9]; p.rough = r[10]; p.subsurface = r[11]; p.ccGloss = r[12];
        p.metallic = r[13]; p.clearcoat = r[14]; p.specTrans = r[15]; p.sheen = r[16];
        const M3 tbn{v3(28), v3(31), v3(34)};
        const V3 wi = v3(22), wo = v3(25);
        const V3 h = norm3(wo + wi);
        float pdf;
        const V3 f = eval_disney(tbn, p, r[17], r[18] != 0.0f, v3(19), wi, wo, h, pdf);
        o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = pdf;
    }
}

void launch_kat(int kind, const float* d_records, uint32_t n, float* d_out, cudaStream_t st) {
    if (n == 0) return;
    k_kat<<<(n + 127) / 128, 128, 0, st>>>(kind, d_records, n, d_out);
}

}  // namespace rt
