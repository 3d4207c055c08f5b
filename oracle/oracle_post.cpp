// ORACLE — test infrastructure only (see oracle_common.h).
//
// CPU restatement of the post-process passes, in float or double:
//   shaders/postprocessing/bloom/blurCommon.h.glsl:10-56 (blurAxis; X pass with the Rec.601 luminance
//   threshold, Y pass without), combine.comp.glsl:15-27 (orig + bloom * intensity) and
//   shaders/postprocessing/tonemap/tonemapping.comp.glsl:17-84 (exp2(exposure), ACES fitted: input
//   matrix, RRT+ODT rational fit, output matrix, clamp to [0, 1]) stored as RGBA8 UNORM (round to
//   nearest; NaN stores 0), in the order of src/Reina.cpp:472-577.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace oracle {

template <class T>
static void blur_axis(const float* in, std::vector<T>& out, int W, int H, bool xaxis, bool threshold_on, T radius, T threshold,
                      const std::vector<T>* src) {
    const int side = xaxis ? W : H;
    const T radius_px = (T)side * radius / (T)100;
    const int K = (int)(radius_px * (T)3 + (T)0.5);
    std::vector<T> w(2 * K + 1);
    T wsum = 0;
    for (int i = -K; i <= K; ++i) {
        const T x = (T)i;
        w[i + K] = std::exp(-x * x / ((T)2 * radius * radius));
        wsum += w[i + K];
    }
    out.assign((size_t)W * H * 4, (T)0);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            T c[3] = {0, 0, 0};
            for (int i = -K; i <= K; ++i) {
                const int cx = xaxis ? x + i : x, cy = xaxis ? y : y + i;
                if (cx < 0 || cx >= W || cy < 0 || cy >= H) continue;
                const size_t q = 4 * ((size_t)cy * W + cx);
                const T p0 = src ? (*src)[q] : (T)in[q], p1 = src ? (*src)[q + 1] : (T)in[q + 1],
                        p2 = src ? (*src)[q + 2] : (T)in[q + 2];
                if (threshold_on) {
                    const T lum = p0 * (T)0.299 + p1 * (T)0.587 + p2 * (T)0.114;
                    if (lum < threshold) continue;
                }
                c[0] += p0 * w[i + K];
                c[1] += p1 * w[i + K];
                c[2] += p2 * w[i + K];
            }
            const size_t o = 4 * ((size_t)y * W + x);
            for (int k = 0; k < 3; ++k) out[o + k] = wsum < (T)0.0001 ? (T)0 : c[k] / wsum;
            out[o + 3] = 1;
        }
}

template <class T>
static T fit(T v) {
    const T a = v * (v + (T)0.0245786) - (T)0.000090537;
    const T b = v * ((T)0.983729 * v + (T)0.4329510) + (T)0.238081;
    return a / b;
}

static uint8_t unorm8(double v) {
    if (std::isnan(v)) return 0;
    v = std::min(std::max(v, 0.0), 1.0);
    return (uint8_t)std::nearbyint(v * 255.0);
}

template <class T>
static void post(const float* accum, int W, int H, T radius, T threshold, T intensity, T exposure, uint8_t* rgba8,
                 float* combined) {
    std::vector<T> ping, pong;
    blur_axis<T>(accum, ping, W, H, true, true, radius, threshold, nullptr);
    blur_axis<T>(accum, pong, W, H, false, false, radius, threshold, &ping);
    const T scale = std::exp2(exposure);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        T r[3];
        for (int k = 0; k < 3; ++k) r[k] = (T)accum[4 * i + k] + pong[4 * i + k] * intensity;
        if (combined) {
            for (int k = 0; k < 3; ++k) combined[4 * i + k] = (float)r[k];
            combined[4 * i + 3] = 1.0f;
        }
        const T c0 = r[0] * scale, c1 = r[1] * scale, c2 = r[2] * scale;
        T v[3] = {c0 * (T)0.59719 + c1 * (T)0.35458 + c2 * (T)0.04823, c0 * (T)0.07600 + c1 * (T)0.90834 + c2 * (T)0.01566,
                  c0 * (T)0.02840 + c1 * (T)0.13383 + c2 * (T)0.83777};
        for (int k = 0; k < 3; ++k) v[k] = fit(v[k]);
        const T o[3] = {v[0] * (T)1.60475 + v[1] * (T)-0.53108 + v[2] * (T)-0.07367,
                        v[0] * (T)-0.10208 + v[1] * (T)1.10813 + v[2] * (T)-0.00605,
                        v[0] * (T)-0.00327 + v[1] * (T)-0.07276 + v[2] * (T)1.07602};
        for (int k = 0; k < 3; ++k) rgba8[4 * i + k] = unorm8((double)o[k]);
        rgba8[4 * i + 3] = 255;
    }
}

}  // namespace oracle

extern "C" void oracle_postprocess(const float* accum, int W, int H, float radius, float threshold, float intensity,
                                   float exposure, int precision, uint8_t* rgba8, float* combined) {
    if (precision == 64)
        oracle::post<double>(accum, W, H, radius, threshold, intensity, exposure, rgba8, combined);
    else
        oracle::post<float>(accum, W, H, radius, threshold, intensity, exposure, rgba8, combined);
}
