// Emissive CDFs on the GPU (Instance::computeCDF, src/scene/Instance.cpp:15-53; duplicate search of
// Instances::computeSamplingDataEmissives, src/scene/Instances.cpp:52-90).
//
// Every arithmetic step is the host build's (Scene::compute_emissive), with explicitly rounded
// intrinsics so that nothing is contracted into an FMA: the vertex transform (row-vector product, as the
// reference's area computation does it), the triangle areas, and the running sums.  The sums are the
// one sequential part: float addition is not associative, so a parallel scan would round differently
// from the reference's loop and move every CDF entry by an ulp or so.  One thread per instance runs the
// loop over precomputed areas instead; everything around it is parallel.
#include "emissive.h"

#include <algorithm>
#include <unordered_map>

#include <cuda_runtime.h>

#include "errors.h"

namespace rt {

namespace {

struct Mat16 {
    float m[16];
};

constexpr int kEmBlock = 256;

// vec4(v, 1) * transform: component c is the dot product with column c, summed left to right.
__global__ void __launch_bounds__(kEmBlock) k_em_transform(const float4* __restrict__ v, size_t nv, Mat16 T,
                                                           float* __restrict__ tv) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
        const float4 p = v[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* col = T.m + 4 * c;
            float s = __fmul_rn(col[0], p.x);
            s = __fadd_rn(s, __fmul_rn(col[1], p.y));
            s = __fadd_rn(s, __fmul_rn(col[2], p.z));
            s = __fadd_rn(s, __fmul_rn(col[3], 1.0f));
            tv[3 * i + c] = s;
        }
    }
}

// |ab x ac| / 2 per triangle.
__global__ void __launch_bounds__(kEmBlock) k_em_area(const float* __restrict__ tv, const uint32_t* __restrict__ idx,
                                                      size_t ntri, float* __restrict__ area) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < ntri; t += (size_t)gridDim.x * blockDim.x) {
        const float* a = tv + 3ull * idx[3 * t + 0];
        const float* b = tv + 3ull * idx[3 * t + 1];
        const float* c = tv + 3ull * idx[3 * t + 2];
        const float ab0 = __fsub_rn(b[0], a[0]), ab1 = __fsub_rn(b[1], a[1]), ab2 = __fsub_rn(b[2], a[2]);
        const float ac0 = __fsub_rn(c[0], a[0]), ac1 = __fsub_rn(c[1], a[1]), ac2 = __fsub_rn(c[2], a[2]);
        const float cr0 = __fsub_rn(__fmul_rn(ab1, ac2), __fmul_rn(ac1, ab2));
        const float cr1 = __fsub_rn(__fmul_rn(ab2, ac0), __fmul_rn(ac2, ab0));
        const float cr2 = __fsub_rn(__fmul_rn(ab0, ac1), __fmul_rn(ac0, ab1));
        const float sq = __fadd_rn(__fadd_rn(__fmul_rn(cr0, cr0), __fmul_rn(cr1, cr1)), __fmul_rn(cr2, cr2));
        area[t] = __fdiv_rn(__fsqrt_rn(sq), 2.0f);
    }
}

// The reference's loop: area += a; cumulative += a * brightness; cdf[t] = cumulative (one thread).
__global__ void k_em_scan(const float* __restrict__ area, size_t ntri, float brightness, float* __restrict__ cdf,
                          float* __restrict__ sums) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    float total = 0.0f, cumulative = 0.0f;
#pragma unroll 8
    for (size_t t = 0; t < ntri; ++t) {
        const float a = area[t];
        total = __fadd_rn(total, a);
        cumulative = __fadd_rn(cumulative, __fmul_rn(a, brightness));
        cdf[t] = cumulative;
    }
    sums[0] = total;
    sums[1] = cumulative;
}

__global__ void __launch_bounds__(kEmBlock) k_em_normalize(float* __restrict__ cdf, size_t ntri,
                                                           const float* __restrict__ sums) {
    const float w = sums[1];
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < ntri; t += (size_t)gridDim.x * blockDim.x)
        cdf[t] = __fdiv_rn(cdf[t], w);
}

// One block per pair of equal-length CDFs: differ[p] = 1 if some |a[e] - b[e]| > tol.
__global__ void __launch_bounds__(kEmBlock) k_em_compare(const float* __restrict__ cdf, const uint64_t* __restrict__ off,
                                                         const uint2* __restrict__ pairs, const uint64_t* __restrict__ len,
                                                         float tol, uint32_t* __restrict__ differ) {
    const uint2 p = pairs[blockIdx.x];
    const float* a = cdf + off[p.x];
    const float* b = cdf + off[p.y];
    const uint64_t n = len[p.x];
    bool d = false;
    for (uint64_t e = threadIdx.x; e < n && !d; e += blockDim.x) d = fabsf(__fsub_rn(a[e], b[e])) > tol;
    if (__syncthreads_or(d) && threadIdx.x == 0) differ[blockIdx.x] = 1u;
}

int grid_for(size_t n) { return (int)std::max<size_t>(1, std::min<size_t>((n + kEmBlock - 1) / kEmBlock, 8192)); }

}  // namespace

void emissive_cdfs_device(int device, const std::vector<EmissiveInput>& in, float tol, std::vector<EmissiveOutput>& out,
                          std::vector<uint8_t>& same) {
    const size_t n = in.size();
    out.assign(n, EmissiveOutput{});
    same.assign(n * n, 0);
    if (n == 0) return;
    check_cuda(cudaSetDevice(device), "cudaSetDevice");
    struct ModelBuffers {
        DeviceBuffer v, idx;
    };
    std::unordered_map<uint32_t, ModelBuffers> models;
    std::vector<uint64_t> off(n + 1, 0);
    size_t max_nv = 0, max_tri = 0;
    for (size_t k = 0; k < n; ++k) {
        off[k + 1] = off[k] + in[k].ntri;
        max_nv = std::max(max_nv, in[k].nv);
        max_tri = std::max(max_tri, in[k].ntri);
        ModelBuffers& m = models[in[k].model];
        if (!m.v.get()) {
            m.v.upload(in[k].vertices, in[k].nv * 4 * sizeof(float));
            m.idx.upload(in[k].indices, in[k].ntri * 3 * sizeof(uint32_t));
        }
    }
    DeviceBuffer cdf(std::max<size_t>(1, off[n]) * sizeof(float)), sums(2 * n * sizeof(float));
    DeviceBuffer tv(std::max<size_t>(1, max_nv) * 3 * sizeof(float)), area(std::max<size_t>(1, max_tri) * sizeof(float));
    cudaStream_t st;
    check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    try {
        for (size_t k = 0; k < n; ++k) {
            const EmissiveInput& e = in[k];
            const ModelBuffers& m = models[e.model];
            Mat16 T;
            std::copy(e.transform, e.transform + 16, T.m);
            float* c = cdf.as<float>() + off[k];
            float* s = sums.as<float>() + 2 * k;
            k_em_transform<<<grid_for(e.nv), kEmBlock, 0, st>>>(m.v.as<float4>(), e.nv, T, tv.as<float>());
            k_em_area<<<grid_for(e.ntri), kEmBlock, 0, st>>>(tv.as<float>(), m.idx.as<uint32_t>(), e.ntri, area.as<float>());
            k_em_scan<<<1, 1, 0, st>>>(area.as<float>(), e.ntri, e.brightness, c, s);
            k_em_normalize<<<grid_for(e.ntri), kEmBlock, 0, st>>>(c, e.ntri, s);
        }
        // duplicate search over every pair of equal triangle count
        std::vector<uint2> pairs;
        for (size_t i = 0; i < n; ++i)
            for (size_t j = i + 1; j < n; ++j)
                if (in[i].ntri == in[j].ntri) pairs.push_back(make_uint2((uint32_t)i, (uint32_t)j));
        std::vector<uint32_t> differ(pairs.size(), 0);
        DeviceBuffer d_pairs, d_off, d_len, d_differ;
        if (!pairs.empty()) {
            std::vector<uint64_t> len(n);
            for (size_t k = 0; k < n; ++k) len[k] = in[k].ntri;
            d_pairs.upload(pairs.data(), pairs.size() * sizeof(uint2));
            d_off.upload(off.data(), n * sizeof(uint64_t));
            d_len.upload(len.data(), n * sizeof(uint64_t));
            d_differ.upload(differ.data(), differ.size() * sizeof(uint32_t));
            for (size_t p0 = 0; p0 < pairs.size(); p0 += 65535) {
                const unsigned blocks = (unsigned)std::min<size_t>(65535, pairs.size() - p0);
                k_em_compare<<<blocks, kEmBlock, 0, st>>>(cdf.as<float>(), d_off.as<uint64_t>(), d_pairs.as<uint2>() + p0,
                                                         d_len.as<uint64_t>(), tol, d_differ.as<uint32_t>() + p0);
            }
        }
        check_cuda(cudaGetLastError(), "emissive CDF kernels");
        std::vector<float> all(off[n]), s(2 * n);
        if (off[n])
            check_cuda(cudaMemcpyAsync(all.data(), cdf.get(), off[n] * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H cdf");
        check_cuda(cudaMemcpyAsync(s.data(), sums.get(), s.size() * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H sums");
        if (!pairs.empty())
            check_cuda(cudaMemcpyAsync(differ.data(), d_differ.get(), differ.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                       st), "D2H differ");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        for (size_t k = 0; k < n; ++k) {
            out[k].cdf.assign(all.begin() + (ptrdiff_t)off[k], all.begin() + (ptrdiff_t)off[k + 1]);
            out[k].area = s[2 * k];
            out[k].weight = s[2 * k + 1];
        }
        for (size_t p = 0; p < pairs.size(); ++p) same[(size_t)pairs[p].x * n + pairs[p].y] = differ[p] ? 0 : 1;
    } catch (...) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        throw;
    }
    cudaStreamDestroy(st);
}

}  // namespace rt
