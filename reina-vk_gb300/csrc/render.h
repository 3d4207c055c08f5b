// Wavefront integrator: host-side workspace and launch sequence.
#pragma once

#include <cstdint>

#include <cuda_runtime_api.h>

#include "device_scene.h"
#include "errors.h"
#include "kernels.h"
#include "../../include/reina/polyglot.h"

namespace rt {

enum RenderMode : uint32_t { kModeReina = 0, kModeNeeMis = 1 };

struct RenderOpts {
    uint32_t width = 0, height = 0;
    uint32_t mode = kModeReina;
    uint32_t seed = 1;
    uint32_t env_mode = 0;          // 0 sky gradient (raytrace.rmiss.glsl), 1 constant colour
    float env_color[3] = {0, 0, 0};
    bool megakernel = false;        // plain form: one kernel, one thread per pixel (no queues)
    bool pass_by_pass = false;      // wavefront one sample pass at a time, direct launches (not the wave engine)
    TraceConfig trace;              // traversal kernels' launch configuration (same images for every setting)
};

// Queue indices of the per-material shade queues (0 = miss, then material_idx + 1).
constexpr int kQueueMiss = 0;
constexpr int kNumQueues = 5;

// Device counters (u32 words): [0], [1] active path queues (ping-pong); [2..6] shade queues; [7] shadow
// queue; [8] error flag; [10..11] rays traced (closest, u64); [12..13] shadow rays traced (u64).
constexpr int kCntActive = 0;
constexpr int kCntQueue = 2;
constexpr int kCntShadow = 7;
constexpr int kCntError = 8;
constexpr int kCntRays = 10;
constexpr int kCntShadowRays = 12;
constexpr int kCntFetchExtend = 14;   // ray-fetch counters of the cooperative extend / shadow kernels
constexpr int kCntFetchShadow = 15;
// Traversal work of the cooperative kernels (u64 each): BVH8 nodes visited and triangles tested by the
// closest-hit (extension) and any-hit (shadow) rays, and the hits shaded by a material kernel.
constexpr int kCntNodes = 16;
constexpr int kCntTris = 18;
constexpr int kCntShadowNodes = 20;
constexpr int kCntShadowTris = 22;
constexpr int kCntShaded = 24;
constexpr int kNumCounters = 26;

// Plain-pointer view of the path state (SoA) passed to every kernel.
struct PathState {
    float *ox, *oy, *oz, *dx, *dy, *dz;      // current ray
    uint32_t* hprim;                          // closest hit of the current ray
    float *hu, *hv;
    float *tr, *tg, *tb;                      // throughput
    float *rr, *rg, *rb;                      // radiance of the current sample
    uint32_t* rng;
    uint32_t* flags;                          // bit 0 insideDielectric, bit 1 previous vertex sampled a light
    float* acc;                               // accumulatedDistance
    float* ppdf;                              // BSDF pdf of the direction sampled at the previous vertex
    // per pixel
    uint32_t* pix_rng;
    float* pix_acc;
    float *sr, *sg, *sb;                      // sum of kept samples
    uint32_t* cnt;                            // kept samples
    // queues
    uint32_t* q_active[2];
    uint32_t* q_shade;                        // kNumQueues x P
    uint32_t* q_shadow;                       // shadow records: path index
    float *s_ox, *s_oy, *s_oz, *s_dx, *s_dy, *s_dz, *s_tmax, *s_cr, *s_cg, *s_cb;
    uint32_t* counters;
};

struct RenderLaunch {
    DeviceScene s;
    RtPushConsts pc;
    PathState ps;
    uint32_t W, H, P;
    uint32_t mode, seed, env_mode;
    float env[3];
    uint32_t sample;          // sample index within the frame (one wave per sample)
    int refill;               // persistent traversal refill threshold
    float* accum;             // W*H*4 RGBA32F (device)
    float* samples;           // optional W*H*spp*3 per-sample colours (device)
};

class RenderWorkspace {
public:
    void ensure(uint32_t paths);
    PathState view() const { return ps_; }
    size_t bytes() const { return buf_.bytes(); }

private:
    DeviceBuffer buf_;
    uint32_t capacity_ = 0;
    PathState ps_{};
};

struct RenderStats {
    uint64_t rays = 0;          // closest-hit rays traced (path segments)
    uint64_t shadow_rays = 0;
    uint64_t nodes = 0, tris = 0, shadow_nodes = 0, shadow_tris = 0, shaded = 0;   // cooperative kernels' counts
    uint32_t error = 0;
};

// Renders one frame (RtPushConsts::samplesPerPixel samples per pixel, running mean with the image when
// sampleBatch > 0) into d_accum.  Enqueued on `st`; if `stats` is given the call synchronizes and
// reads the counters; if `err_accum` is given, the frame's device error flags are OR-ed into that word
// on `st` after the frame (the asynchronous entry points' error word, read by reina_ctx_device_error).
void render_frame(RenderWorkspace& ws, const DeviceScene& s, const RtPushConsts& pc, const RenderOpts& opt,
                  float* d_accum, float* d_samples, int sm_count, cudaStream_t st, RenderStats* stats,
                  uint32_t* err_accum = nullptr);

// The same frame with the path state in a fixed device array of the library (no allocation); at most
// kNoAllocMaxPixels pixels.  `device` must be the current device.
constexpr uint32_t kNoAllocMaxPixels = 65536;
constexpr int kNoAllocMaxDevices = 64;
void render_frame_noalloc(int device, const DeviceScene& s, const RtPushConsts& pc, const RenderOpts& opt,
                          float* d_accum, float* d_samples, int sm_count, cudaStream_t st, uint32_t* err_accum);

}  // namespace rt
