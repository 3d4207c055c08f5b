// Post-process kernels: bloom (shaders/postprocessing/bloom/{blurCommon.h,blurX.comp,blurY.comp,
// combine.comp}.glsl) and tone mapping (shaders/postprocessing/tonemap/tonemapping.comp.glsl), run in
// the order of Reina::applyBloom / applyTonemapping (src/Reina.cpp:472-577):
//   blurX(accum -> ping, with threshold)  blurY(ping -> pong)  combine(accum, pong -> ping)  tonemap(ping -> rgba8)
// All taps of the reference's kernel are summed (kernelSize = int(radiusPx * 3 + 0.5) on each side), so a
// NaN pixel spreads exactly as it does there; the Gaussian weights and their sum (which counts
// out-of-image and thresholded taps, blurCommon.h.glsl:24-31) are computed once per pass.
#include <cuda_runtime.h>

#include <cmath>

#include "post.h"

namespace rt {

constexpr int kPostBlock = 256;

// gauss(x, sigma) = exp(-x^2 / (2 sigma^2)) for x = -K..K, and their float sum in that order.
__global__ void k_bloom_weights(float* w, int K, float sigma) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    float sum = 0.0f;
    for (int i = -K; i <= K; ++i) {
        const float x = (float)i;
        const float g = expf(-x * x / (2.0f * sigma * sigma));
        w[i + K] = g;
        sum += g;
    }
    w[2 * K + 1] = sum;
}

template <bool X>
__global__ void __launch_bounds__(kPostBlock) k_blur(const float4* __restrict__ in, float4* __restrict__ out, int W, int H,
                                                     const float* __restrict__ wts, int K, float threshold) {
    const int n = W * H;
    const float wsum = wts[2 * K + 1];
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int x = idx % W, y = idx / W;
        float cr = 0.0f, cg = 0.0f, cb = 0.0f;
        for (int i = -K; i <= K; ++i) {
            const int cx = X ? x + i : x;
            const int cy = X ? y : y + i;
            if (cx < 0 || cx >= W || cy < 0 || cy >= H) continue;
            const float4 p = __ldg(in + (size_t)cy * W + cx);
            if (X) {
                const float lum = p.x * 0.299f + p.y * 0.587f + p.z * 0.114f;
                if (lum < threshold) continue;
            }
            const float wgt = wts[i + K];
            cr += p.x * wgt;
            cg += p.y * wgt;
            cb += p.z * wgt;
        }
        if (wsum < 0.0001f) {
            cr = cg = cb = 0.0f;
        } else {
            cr /= wsum;
            cg /= wsum;
            cb /= wsum;
        }
        out[idx] = make_float4(cr, cg, cb, 1.0f);
    }
}

// combine.comp.glsl:15-27 then tonemapping.comp.glsl:66-84 (exposure, ACES fitted, clamp, RGBA8 UNORM).
__device__ __forceinline__ uint8_t to_unorm8(float v) {
    if (!(v == v)) return 0;   // NaN stores as 0
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return (uint8_t)__float2uint_rn(v * 255.0f);
}

__device__ __forceinline__ float3 aces_fitted(float3 c) {
    // color * ACESInputMat: GLSL row vector times a matrix built from columns -> dot with each column
    float3 v = make_float3(c.x * 0.59719f + c.y * 0.35458f + c.z * 0.04823f, c.x * 0.07600f + c.y * 0.90834f + c.z * 0.01566f,
                           c.x * 0.02840f + c.y * 0.13383f + c.z * 0.83777f);
    auto fit = [](float x) {
        const float a = x * (x + 0.0245786f) - 0.000090537f;
        const float b = x * (0.983729f * x + 0.4329510f) + 0.238081f;
        return a / b;
    };
    v = make_float3(fit(v.x), fit(v.y), fit(v.z));
    float3 o = make_float3(v.x * 1.60475f + v.y * -0.53108f + v.z * -0.07367f, v.x * -0.10208f + v.y * 1.10813f + v.z * -0.00605f,
                           v.x * -0.00327f + v.y * -0.07276f + v.z * 1.07602f);
    return o;
}

__global__ void __launch_bounds__(kPostBlock) k_combine_tonemap(const float4* __restrict__ orig, const float4* __restrict__ bloom,
                                                                float4* __restrict__ combined, uchar4* __restrict__ out, int n,
                                                                float intensity, float exposure_scale) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 o = orig[i];
        const float4 b = bloom[i];
        const float3 r = make_float3(o.x + b.x * intensity, o.y + b.y * intensity, o.z + b.z * intensity);
        if (combined) combined[i] = make_float4(r.x, r.y, r.z, 1.0f);
        const float3 t = aces_fitted(make_float3(r.x * exposure_scale, r.y * exposure_scale, r.z * exposure_scale));
        out[i] = make_uchar4(to_unorm8(t.x), to_unorm8(t.y), to_unorm8(t.z), 255);
    }
}

void PostWorkspace::ensure(size_t pixels, int k) {
    if (pixels > cap_px_) {
        ping.alloc(pixels * sizeof(float4));
        pong.alloc(pixels * sizeof(float4));
        cap_px_ = pixels;
    }
    if ((size_t)(2 * k + 2) > cap_w_) {
        weights.alloc((2 * (size_t)k + 2) * sizeof(float));
        cap_w_ = 2 * (size_t)k + 2;
    }
}

static int bloom_kernel_size(int side, float radius) {
    const float radius_px = (float)side * radius / 100.0f;   // blurCommon.h.glsl:19
    return (int)(radius_px * 3.0f + 0.5f);
}

void postprocess(PostWorkspace& ws, const float* d_accum, int W, int H, const BloomPushConsts& bloom,
                 const TonemappingPushConsts& tm, uint8_t* d_rgba8, float* d_combined, int sm_count, cudaStream_t st) {
    const size_t n = (size_t)W * H;
    if (n == 0) return;
    const int kx = bloom_kernel_size(W, bloom.radius);
    const int ky = bloom_kernel_size(H, bloom.radius);
    if (kx < 0 || ky < 0 || kx > (1 << 20) || ky > (1 << 20)) fail(REINA_ERR_INVALID, "bloom radius out of range");
    ws.ensure(n, std::max(kx, ky));
    const int blocks = (int)std::min<size_t>((n + kPostBlock - 1) / kPostBlock, (size_t)std::max(1, sm_count) * 16);
    float* w = ws.weights.as<float>();
    k_bloom_weights<<<1, 1, 0, st>>>(w, kx, bloom.radius);
    k_blur<true><<<blocks, kPostBlock, 0, st>>>(reinterpret_cast<const float4*>(d_accum), ws.ping.as<float4>(), W, H, w, kx,
                                                bloom.threshold);
    k_bloom_weights<<<1, 1, 0, st>>>(w, ky, bloom.radius);
    k_blur<false><<<blocks, kPostBlock, 0, st>>>(ws.ping.as<float4>(), ws.pong.as<float4>(), W, H, w, ky, 0.0f);
    const float scale = exp2f(tm.exposure);
    k_combine_tonemap<<<blocks, kPostBlock, 0, st>>>(reinterpret_cast<const float4*>(d_accum), ws.pong.as<float4>(),
                                                     reinterpret_cast<float4*>(d_combined), reinterpret_cast<uchar4*>(d_rgba8),
                                                     (int)n, bloom.intensity, scale);
    check_cuda(cudaGetLastError(), "postprocess launch");
}

}  // namespace rt
