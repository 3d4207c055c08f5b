// ORACLE — test infrastructure only (see oracle_common.h).
//
// CPU restatement, templated on the scalar type, of the reference's shading math:
//   shaders/raytrace/brdfDisney.h.glsl (GGX VNDF sampling, aniso D, Smith G, GTR1 clearcoat, Burley
//   diffuse + subsurface, sheen, rough glass, sampleDisney / evalDisney), closestHitCommon.h.glsl
//   (randomUnitVec, fuzzyReflection, diffuseReflection, offsetPositionAlongNormal) and pdf.h.glsl.
// GLSL built-ins follow the GLSL 4.60 specification: reflect(I, N) = I - 2 dot(N, I) N; refract returns
// the zero vector when k < 0; faceforward(N, I, Nref) = dot(Nref, I) < 0 ? N : -N; mix(x, y, a) =
// x (1 - a) + y a; mod(x, y) = x - y floor(x / y).  pow(x, n) with a literal integer n is evaluated as
// repeated multiplication (GLSL leaves pow of a negative base undefined; the reference's renders show
// the squared terms of brdfDisney.h.glsl evaluating as squares).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "oracle_common.h"

namespace oracle {

template <class T> inline T kpi() { return (T)3.14159265; }      // k_pi, shaderCommon.h.glsl:47
template <class T> inline T kinvpi() { return (T)0.31830989; }   // k_inv_pi, shaderCommon.h.glsl:48

template <class T> inline T sq(T x) { return x * x; }
template <class T> inline T pow5(T x) { return x * x * x * x * x; }

template <class T>
struct Mat3 {   // columns c0, c1, c2 (GLSL mat3(c0, c1, c2))
    Vec3<T> c0, c1, c2;
};
template <class T> inline Vec3<T> mul(const Mat3<T>& m, Vec3<T> v) { return m.c0 * v.x + m.c1 * v.y + m.c2 * v.z; }
template <class T> inline Vec3<T> mulT(const Mat3<T>& m, Vec3<T> v) { return Vec3<T>(dot(m.c0, v), dot(m.c1, v), dot(m.c2, v)); }

template <class T> inline Vec3<T> reflect(Vec3<T> I, Vec3<T> N) { return I - N * ((T)2 * dot(N, I)); }
template <class T> inline Vec3<T> refract(Vec3<T> I, Vec3<T> N, T eta) {
    const T d = dot(N, I);
    const T k = (T)1 - eta * eta * ((T)1 - d * d);
    if (k < (T)0) return Vec3<T>((T)0, (T)0, (T)0);
    return I * eta - N * (eta * d + std::sqrt(k));
}
template <class T> inline Vec3<T> faceforward(Vec3<T> N, Vec3<T> I, Vec3<T> Nref) { return dot(Nref, I) < (T)0 ? N : -N; }
template <class T> inline T mixs(T x, T y, T a) { return x * ((T)1 - a) + y * a; }
template <class T> inline Vec3<T> mixv(Vec3<T> x, Vec3<T> y, T a) { return x * ((T)1 - a) + y * a; }
template <class T> inline Vec3<T> mixv(Vec3<T> x, Vec3<T> y, Vec3<T> a) {
    return Vec3<T>(mixs(x.x, y.x, a.x), mixs(x.y, y.y, a.y), mixs(x.z, y.z, a.z));
}
template <class T> inline T clampT(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }

// ---- closestHitCommon.h.glsl:195-222 ---------------------------------------------------------------
template <class T>
inline Vec3<T> randomUnitVec(uint32_t& rng) {
    for (;;) {   // 3 draws per try, accept 1e-4 < |v|^2 < 1
        const T a = rng_random<T>(rng), b = rng_random<T>(rng), c = rng_random<T>(rng);
        const Vec3<T> v(a * (T)2 - (T)1, b * (T)2 - (T)1, c * (T)2 - (T)1);
        const T l2 = dot(v, v);
        if ((T)0.0001 < l2 && l2 < (T)1) return normalize(v);
    }
}
template <class T>
inline Vec3<T> fuzzyReflection(Vec3<T> rayIn, Vec3<T> n, T fuzz, uint32_t& rng) {
    return reflect(normalize(rayIn), normalize(n)) + randomUnitVec<T>(rng) * fuzz;
}
template <class T>
inline Vec3<T> diffuseReflection(Vec3<T> n, uint32_t& rng) {
    const T theta = (T)2 * kpi<T>() * rng_random<T>(rng);
    const T u = (T)2 * rng_random<T>(rng) - (T)1;
    const T r = std::sqrt((T)1 - u * u);
    return normalize(n + Vec3<T>(r * std::cos(theta), r * std::sin(theta), u));
}

// Wächter & Binder, "A Fast and Robust Method for Avoiding Self-Intersection" (Ray Tracing Gems 2019),
// as in closestHitCommon.h.glsl:156-177; the float bit pattern is offset in both precisions (the
// double mode applies the float-space offset to the position rounded to float).
template <class T>
inline Vec3<T> offsetAlongNormal(Vec3<T> p, Vec3<T> n) {
    Vec3<T> out;
    for (int k = 0; k < 3; ++k) {
        const float pk = (float)p[k];
        const int of = (int)((float)256.0f * (float)n[k]);
        int32_t bits;
        std::memcpy(&bits, &pk, 4);
        bits += (pk < 0.0f) ? -of : of;
        float pi;
        std::memcpy(&pi, &bits, 4);
        const T near0 = p[k] + (T)(1.0 / 65536.0) * n[k];
        out[k] = std::fabs(p[k]) < (T)(1.0 / 32.0) ? near0 : (sizeof(T) == 4 ? (T)pi : (T)pi + (p[k] - (T)pk));
    }
    return out;
}

// dielectric.rchit.glsl:14-38 / disney.rchit.glsl:10-34
template <class T>
inline Vec3<T> offsetForDielectric(Vec3<T> p, Vec3<T> n, Vec3<T> dir) {
    return offsetAlongNormal(p, dot(n, dir) < (T)0 ? -n : n);
}

template <class T> inline T pdfLambertian(Vec3<T> n, Vec3<T> w) { return std::max(dot(n, w), (T)0) / kpi<T>(); }
template <class T> inline T powerHeuristic(T a, T b) { return a * a / (a * a + b * b); }   // pdf.h.glsl:4-7

// ---- brdfDisney.h.glsl ------------------------------------------------------------------------------
template <class T>
inline Vec3<T> sampleGGXVNDF(Vec3<T> V, T ax, T ay, uint32_t& rng) {   // :9-40
    const bool flip = V.z < (T)0;
    if (flip) V.z = -V.z;
    const T r1 = rng_random<T>(rng), r2 = rng_random<T>(rng);
    const Vec3<T> Vh = normalize(Vec3<T>(ax * V.x, ay * V.y, V.z));
    const T lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    const Vec3<T> T1 = lensq > (T)0 ? Vec3<T>(-Vh.y, Vh.x, (T)0) * ((T)1 / std::sqrt(lensq)) : Vec3<T>((T)1, (T)0, (T)0);
    const Vec3<T> T2 = cross(Vh, T1);
    const T r = std::sqrt(r1);
    const T phi = (T)2 * kpi<T>() * r2;
    const T t1 = r * std::cos(phi);
    T t2 = r * std::sin(phi);
    const T s = (T)0.5 * ((T)1 + Vh.z);
    t2 = ((T)1 - s) * std::sqrt((T)1 - t1 * t1) + s * t2;
    Vec3<T> Nh = T1 * t1 + T2 * t2 + Vh * std::sqrt(std::max((T)0, (T)1 - t1 * t1 - t2 * t2));
    if (flip) Nh.z = -Nh.z;
    return normalize(Vec3<T>(ax * Nh.x, ay * Nh.y, std::max((T)0, Nh.z)));
}

template <class T>
inline T D_GGX_Aniso(Vec3<T> m, T ax, T ay) {   // :42-48
    const T NoM = std::max(m.z, (T)0);
    const T inv = (T)1 / ((m.x / ax) * (m.x / ax) + (m.y / ay) * (m.y / ay) + NoM * NoM);
    return inv * inv / (kpi<T>() * ax * ay);
}

template <class T>
inline T pdfGGXReflection(Vec3<T> i, Vec3<T> o, T ax, T ay) {   // :55-73
    const Vec3<T> m = normalize(i + o);
    const T ndf = D_GGX_Aniso(m, ax, ay);
    const T aix = ax * i.x, aiy = ay * i.y;
    const T len2 = aix * aix + aiy * aiy;
    const T t = std::sqrt(len2 + i.z * i.z);
    if (i.z >= (T)0) {
        const T a = clampT(std::min(ax, ay), (T)0, (T)1);
        const T s = (T)1 + std::sqrt(i.x * i.x + i.y * i.y);
        const T a2 = a * a, s2 = s * s;
        const T k = ((T)1 - a2) * s2 / (s2 + a2 * i.z * i.z);
        return ndf / ((T)2 * (k * i.z + t));
    }
    return ndf * (t - i.z) / ((T)2 * len2);
}

template <class T>
inline Vec3<T> sampleGTR1_attempt2(T alpha, uint32_t& rng) {   // :96-111
    const T r1 = rng_random<T>(rng), r2 = rng_random<T>(rng);
    const T a = std::max((T)0.001, alpha);
    const T cosh_el = std::sqrt(((T)1 - std::exp(r1 * std::log(a * a))) / ((T)1 - a * a));
    const T h_el = std::acos(cosh_el);
    const T h_az = (T)2 * kpi<T>() * r2;
    return Vec3<T>(std::sin(h_el) * std::cos(h_az), std::sin(h_el) * std::sin(h_az), cosh_el);
}

template <class T> inline T FD(Vec3<T> n, Vec3<T> w, T fd90) {   // :128-131
    return (T)1 + (fd90 - (T)1) * pow5((T)1 - std::max(dot(n, w), (T)0));
}

template <class T>
inline Vec3<T> evalDiffuse(T roughness, T subsurface, Vec3<T> base, Vec3<T> n, Vec3<T> wi, Vec3<T> wo, Vec3<T> h) {
    // fBaseDiffuse (:154-161) mixed with fSubsurface (:141-152) by `subsurface` (:163-168)
    const T hwo = dot(h, wo);
    const T fd90 = (T)0.5 + (T)2 * roughness * std::max(hwo, (T)0) * std::max(hwo, (T)0);
    const Vec3<T> baseDiffuse = base / kpi<T>() * FD(n, wi, fd90) * FD(n, wo, fd90);
    const Vec3<T> k = base * (T)1.25 * kinvpi<T>();
    const T fss90 = roughness * std::max(dot(h, wo), (T)0) * std::max(dot(h, wo), (T)0);
    const T fssIn = (T)1 + (fss90 - (T)1) * pow5((T)1 - std::max(dot(n, wi), (T)0));
    const T fssOut = (T)1 + (fss90 - (T)1) * pow5((T)1 - std::max(dot(n, wo), (T)0));
    const T third = (T)1 / (std::max(dot(n, wi), (T)0) + std::max(dot(n, wo), (T)0)) - (T)0.5;
    const Vec3<T> fsub = k * (fssIn * fssOut * third + (T)0.5);
    return mixv(baseDiffuse, fsub, subsurface);
}

template <class T> inline T pdfDiffuse(Vec3<T> wo, Vec3<T> n) {   // :170-179
    const T c = dot(n, wo);
    return c <= (T)0 ? (T)0 : c * kinvpi<T>();
}

template <class T>
inline Vec3<T> sampleDiffuse(Vec3<T> n, uint32_t& rng) {   // :181-201
    const T xi1 = rng_random<T>(rng), xi2 = rng_random<T>(rng);
    const T r = std::sqrt(xi1);
    const T phi = (T)2 * kpi<T>() * xi2;
    const T x = r * std::cos(phi), y = r * std::sin(phi);
    const T z = std::sqrt(std::max((T)0, (T)1 - xi1));
    const Vec3<T> t = std::fabs(n.x) < (T)0.5 ? normalize(cross(n, Vec3<T>((T)1, (T)0, (T)0)))
                                             : normalize(cross(n, Vec3<T>((T)0, (T)1, (T)0)));
    const Vec3<T> b = cross(n, t);
    return normalize(t * x + b * y + n * z);
}

template <class T> inline T evalR0(T ior) { return (ior - (T)1) * (ior - (T)1) / ((ior + (T)1) * (ior + (T)1)); }
template <class T> inline T luminance(Vec3<T> c) { return dot(c, Vec3<T>((T)0.2126, (T)0.7152, (T)0.0722)); }

template <class T>
inline Vec3<T> evalFm(Vec3<T> base, Vec3<T> h, Vec3<T> wo, T specular, Vec3<T> specTint, T metallic, T eta) {   // :215-222
    const T lum = luminance(base);
    const Vec3<T> one((T)1, (T)1, (T)1);
    const Vec3<T> ctint = lum > (T)0 ? base / lum : one;
    const Vec3<T> ks = (one - ctint) + specTint * ctint;
    const Vec3<T> c0 = ks * (specular * evalR0(eta) * ((T)1 - metallic)) + base * metallic;
    return c0 + (one - c0) * pow5((T)1 - std::fabs(dot(h, wo)));
}

template <class T> inline T evalDm(Vec3<T> hl, T ax, T ay) {   // :224-229
    const T c = kpi<T>() * ax * ay;
    const T o = sq(sq(hl.x) / sq(ax) + sq(hl.y) / sq(ay) + sq(hl.z));
    return (T)1 / (c * o);
}
template <class T> inline T lambda(Vec3<T> wl, T ax, T ay) {   // :231-234
    const T s = std::sqrt((T)1 + (sq(wl.x * ax) + sq(wl.y * ay)) / sq(wl.z));
    return (s - (T)1) / (T)2;
}
template <class T> inline T smithG(Vec3<T> wl, T ax, T ay) { return (T)1 / ((T)1 + lambda(wl, ax, ay)); }
template <class T> inline T evalGm(Vec3<T> wi, Vec3<T> wo, T ax, T ay) { return smithG(wi, ax, ay) * smithG(wo, ax, ay); }

template <class T> inline void alphas(T aniso, T rough, T& ax, T& ay) {
    const T aspect = std::sqrt((T)1 - (T)0.9 * aniso);
    ax = std::max((T)0.0001, rough * rough / aspect);
    ay = std::max((T)0.0001, rough * rough * aspect);
}

template <class T>
inline Vec3<T> evalMetal(const Mat3<T>& tbn, Vec3<T> base, T aniso, T rough, Vec3<T> n, Vec3<T> wi, Vec3<T> wo,
                         Vec3<T> h, T specular, Vec3<T> specTint, T metallic, T eta) {   // :247-267
    T ax, ay;
    alphas(aniso, rough, ax, ay);
    const Vec3<T> fm = evalFm(base, h, wo, specular, specTint, metallic, eta);
    const Vec3<T> wiT = normalize(mulT(tbn, wi)), woT = normalize(mulT(tbn, wo)), hT = normalize(mulT(tbn, h));
    const T dm = evalDm(hT, ax, ay);
    const T gm = evalGm(wiT, woT, ax, ay);
    const T ni = std::fabs(dot(n, wi)), no = std::fabs(dot(n, wo));
    return fm * dm * gm / ((T)4 * ni * no);
}

template <class T>
inline Vec3<T> sampleMetal(const Mat3<T>& tbn, T aniso, T rough, Vec3<T> wi, uint32_t& rng) {   // :269-285
    T ax, ay;
    alphas(aniso, rough, ax, ay);
    Vec3<T> h = sampleGGXVNDF(mulT(tbn, wi), ax, ay, rng);
    h = normalize(mul(tbn, h));
    return reflect(-wi, h);
}

template <class T>
inline T pdfMetal(const Mat3<T>& tbn, Vec3<T> wi, Vec3<T> wo, T aniso, T rough) {   // :287-299
    T ax, ay;
    alphas(aniso, rough, ax, ay);
    return pdfGGXReflection(mulT(tbn, wi), mulT(tbn, wo), ax, ay);
}

template <class T> inline T sepSmithG1(Vec3<T> w, T a) {   // :313-319
    const T a2 = a * a;
    return (T)2 / ((T)1 + std::sqrt(a2 + ((T)1 - a2) * w.z * w.z));
}
template <class T> inline T evalDc(T ag, Vec3<T> hl) {   // :328-333
    return (ag * ag - (T)1) / (kpi<T>() * std::log(ag * ag) * ((T)1 + (ag * ag - (T)1) * (hl.z * hl.z)));
}
template <class T> inline T clearcoatAlpha(T gloss) { return ((T)1 - gloss) * (T)0.1 + gloss * (T)0.001; }

template <class T>
inline Vec3<T> evalClearcoat(const Mat3<T>& tbn, Vec3<T> wi, Vec3<T> wo, T gloss, Vec3<T> h) {   // :341-354
    const T ag = clearcoatAlpha(gloss);
    const Vec3<T> hT = mulT(tbn, h), wiT = mulT(tbn, wi), woT = mulT(tbn, wo);
    const T r0 = evalR0((T)1.5);
    const T fc = r0 + ((T)1 - r0) * pow5((T)1 - dot(h, wo));
    const T gc = sepSmithG1(wiT, (T)0.25) * sepSmithG1(woT, (T)0.25);
    const T dc = evalDc(ag, hT);
    const T v = (T)0.25 * fc * gc * dc;
    return Vec3<T>(v, v, v);
}

template <class T>
inline Vec3<T> sampleClearcoat(const Mat3<T>& tbn, T gloss, Vec3<T> wi, uint32_t& rng) {   // :356-366
    Vec3<T> h = normalize(sampleGTR1_attempt2(clearcoatAlpha(gloss), rng));
    h = normalize(mul(tbn, h));
    return normalize(reflect(-wi, h));
}

template <class T>
inline T pdfClearcoat(const Mat3<T>& tbn, Vec3<T> wi, Vec3<T> wo, Vec3<T> h, T gloss) {   // :368-383
    const T ag = clearcoatAlpha(gloss);
    const Vec3<T> wiT = mulT(tbn, wi), woT = mulT(tbn, wo), hT = mulT(tbn, h);
    if (wiT.z <= (T)0 || woT.z <= (T)0) return (T)0;
    const T dc = evalDc(ag, hT) * hT.z;
    return dc / ((T)4 * std::fabs(dot(woT, hT)));
}

template <class T> inline T reflectance(T cosine, T ri) {   // :389-394, dielectric.rchit.glsl:7-12
    T r0 = ((T)1 - ri) / ((T)1 + ri);
    r0 = r0 * r0;
    return r0 + ((T)1 - r0) * pow5((T)1 - cosine);
}

template <class T>
inline Vec3<T> sampleGlass(const Mat3<T>& tbn, Vec3<T> wi, T rough, T aniso, T eta, uint32_t& rng, bool& refracted) {   // :396-431
    T ax, ay;
    alphas(aniso, rough, ax, ay);
    const Vec3<T> wiT = mulT(tbn, wi);
    const Vec3<T> hT = sampleGGXVNDF(wiT, ax, ay, rng);
    const T cosT = dot(wiT, hT);
    const Vec3<T> hW = normalize(mul(tbn, hT));
    const T refl = reflectance(cosT, eta);
    const T sinT = std::sqrt((T)1 - cosT * cosT);
    const bool cannot = eta * sinT > (T)1;
    if (cannot || refl > rng_random<T>(rng)) {
        refracted = false;
        return reflect(-wi, hW);
    }
    refracted = true;
    return refract(-wi, hW, eta);
}

template <class T> inline T SmithGAniso(T NdV, T VdX, T VdY, T ax, T ay) {   // :433-439
    const T a = VdX * ax, b = VdY * ay, c = NdV;
    return ((T)2 * NdV) / (NdV + std::sqrt(a * a + b * b + c * c));
}

template <class T>
inline Vec3<T> evalMicrofacetRefraction(Vec3<T> base, T aniso, T rough, T eta, Vec3<T> V, Vec3<T> L, Vec3<T> H, T& pdf) {   // :441-467
    T ax, ay;
    alphas(aniso, rough, ax, ay);
    pdf = (T)0;
    if (L.z >= (T)0) return Vec3<T>((T)0, (T)0, (T)0);
    const T LdH = dot(L, H), VdH = dot(V, H);
    const T D = evalDm(H, ax, ay);
    const T G1 = SmithGAniso(std::fabs(V.z), V.x, V.y, ax, ay);
    const T G2 = G1 * SmithGAniso(std::fabs(L.z), L.x, L.y, ax, ay);
    T denom = LdH + VdH * eta;
    denom *= denom;
    const T jac = std::fabs(LdH) * (eta * eta) / denom;
    pdf = G1 * std::max((T)0, VdH) * D * jac / V.z;
    const T F = reflectance(dot(V, H), eta);
    const Vec3<T> sb(std::sqrt(base.x), std::sqrt(base.y), std::sqrt(base.z));
    return sb * (((T)1 - F) * D * G2 * std::fabs(VdH) * jac / std::fabs(L.z * V.z));
}

template <class T>
inline Vec3<T> glass(const Mat3<T>& tbn, Vec3<T> base, T aniso, T rough, T eta, Vec3<T> n, Vec3<T> wi, Vec3<T> wo,
                     bool didRefract, T& pdf) {   // :539-581
    Vec3<T> h = didRefract ? normalize(wo + wi * eta) : normalize(wo + wi);
    if (dot(h, n) < (T)0) h = -h;
    T tpdf;
    const Vec3<T> gf = evalMicrofacetRefraction(base, aniso, rough, eta, mulT(tbn, wi), mulT(tbn, wo), mulT(tbn, h), tpdf);
    const T mpdf = pdfMetal(tbn, wi, wo, aniso, rough);
    const Vec3<T> mf = evalMetal(tbn, base, aniso, rough, n, wi, wo, h, (T)0, Vec3<T>((T)1, (T)1, (T)1), (T)1, eta);
    if (didRefract) { pdf = tpdf; return gf; }
    pdf = mpdf;
    return mf;
}

template <class T>
inline Vec3<T> evalSheen(Vec3<T> base, Vec3<T> wo, Vec3<T> h, Vec3<T> n, Vec3<T> sheenTint) {   // :587-594
    const T lum = luminance(base);
    const Vec3<T> one((T)1, (T)1, (T)1);
    const Vec3<T> ctint = lum > (T)0 ? base / lum : one;
    const Vec3<T> cs = mixv(one, ctint, sheenTint);
    return cs * (pow5((T)1 - std::max(dot(h, wo), (T)0)) * std::max(dot(n, wo), (T)0));
}

template <class T>
struct DisneyParams {
    Vec3<T> base, specTint, sheenTint;
    T aniso, rough, subsurface, ccGloss, metallic, clearcoat, specTrans, sheen;
};

template <class T>
inline Vec3<T> sampleDisney(const Mat3<T>& tbn, const DisneyParams<T>& p, T eta, Vec3<T> n, Vec3<T> wi, bool& didRefract,
                            bool& choseGlass, uint32_t& rng) {   // :609-654
    const T dw = ((T)1 - p.specTrans) * ((T)1 - p.metallic);
    const T mw = p.metallic;
    const T cw = (T)0.25 * p.clearcoat;
    const T gw = ((T)1 - p.metallic) * p.specTrans;
    const T c0 = dw, c1 = c0 + mw, c2 = c1 + cw, c3 = c2 + gw;
    didRefract = false;
    const T r = rng_random<T>(rng) * c3;
    choseGlass = false;
    if (r < c0) return sampleDiffuse(n, rng);
    if (r < c1) return sampleMetal(tbn, p.aniso, p.rough, wi, rng);
    if (r < c2) return sampleClearcoat(tbn, p.ccGloss, wi, rng);
    choseGlass = true;
    return sampleGlass(tbn, wi, p.rough, p.aniso, eta, rng, didRefract);
}

template <class T>
inline Vec3<T> evalDisney(const Mat3<T>& tbn, const DisneyParams<T>& p, T eta, bool didRefract, Vec3<T> n, Vec3<T> wi,
                          Vec3<T> wo, Vec3<T> h, T& pdf) {   // :656-711
    const T dw = ((T)1 - p.specTrans) * ((T)1 - p.metallic);
    const T mw = p.metallic;
    const T cw = (T)0.25 * p.clearcoat;
    const T gw = ((T)1 - p.metallic) * p.specTrans;
    const T sum = dw + mw + gw;
    const Vec3<T> fd = evalDiffuse(p.rough, p.subsurface, p.base, n, wi, wo, h);
    const T dpdf = pdfDiffuse(wo, n);
    const Vec3<T> fs = evalSheen(p.base, wo, h, n, p.sheenTint);
    // the specular argument of evalMetal receives specularTransmission (:692)
    const Vec3<T> fm = evalMetal(tbn, p.base, p.aniso, p.rough, n, wi, wo, h, p.specTrans, p.specTint, p.metallic, eta);
    const T mpdf = pdfMetal(tbn, wi, wo, p.aniso, p.rough);
    const Vec3<T> fc = evalClearcoat(tbn, wi, wo, p.ccGloss, h);
    const T cpdf = pdfClearcoat(tbn, wi, wo, h, p.ccGloss);
    T gpdf;
    const Vec3<T> fg = glass(tbn, p.base, p.aniso, p.rough, eta, n, wi, wo, didRefract, gpdf);
    pdf = dpdf * dw / sum + mpdf * mw / sum + cpdf * cw + gpdf * gw / sum;
    return (fd + fs * p.sheen) * (dw / sum) + fm * (mw / sum) + fc * cw + fg * (gw / sum);
}

}  // namespace oracle
