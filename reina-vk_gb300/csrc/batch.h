// Multi-job wavefront engine: many scenes, resolutions and sample budgets traced together in shared
// waves.  Used by reina_render_batch (all jobs known up front) and by the request server (jobs join
// and leave between waves).
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include <cuda_runtime_api.h>

#include "device_scene.h"
#include "errors.h"
#include "render.h"
#include "../../include/reina/polyglot.h"

namespace rt {

constexpr uint32_t kMaxWaveSegments = 1024;

// Per-job data the kernels read (one table per wave, holding the jobs present in that wave).
struct JobGpu {
    DeviceScene s;
    RtPushConsts pc;
    uint32_t W, H, mode, seed, env_mode, spp, max_bounces, pad;
    float env[3];
    float pad2;
    float* accum;            // W*H RGBA32F
    float* samples;          // optional W*H*spp*3
    uint32_t* pix_rng;       // per-pixel state: carried RNG, accumulatedDistance, sample sums, count
    float* pix_acc;
    float *sr, *sg, *sb;
    uint32_t* cnt;
};

// A run of wave slots [wave_start, wave_start + count) holding pixels [pixel_start, ...) of one job's
// sample `sample`.
struct WaveSeg {
    uint32_t job;            // index into the wave's job table
    uint32_t wave_start;
    uint32_t pixel_start;
    uint32_t count;
    uint32_t sample;
    uint32_t pad[3];
};

struct WaveHeader {
    uint32_t count;          // paths in the wave
    uint32_t nseg;
    uint32_t njobs;
    uint32_t max_bounces;    // segments to run (max over the wave's jobs)
};

// Host-side description of one job.
struct BatchJob {
    DeviceScene scene;
    RtPushConsts pc;
    RenderOpts opt;
    float* d_accum = nullptr;
    float* d_samples = nullptr;
    // progress
    uint64_t cursor = 0;     // next (sample * W*H + pixel) to schedule
    uint64_t total = 0;      // spp * W*H
    DeviceBuffer pixel_state;
    bool resolved = false;
};

class BatchEngine {
public:
    BatchEngine(int device, int sm_count, uint32_t wave_capacity, bool use_graphs,
                const TraceConfig& trace = TraceConfig());
    ~BatchEngine();
    BatchEngine(const BatchEngine&) = delete;
    BatchEngine& operator=(const BatchEngine&) = delete;

    // Allocates the job's per-pixel state (24 bytes per pixel); the job must outlive its waves.
    static void prepare(BatchJob& job);
    // Packs the next wave from `jobs` (fair share of the capacity, oldest first for leftovers; with
    // `fifo`, each job in order takes all it can use), runs it and resolves the jobs it completes.
    // Returns the number of paths traced (0 = nothing to do).  Synchronizes the stream at the end.
    uint64_t run_wave(const std::vector<BatchJob*>& jobs, cudaStream_t st, bool fifo = false);
    uint32_t capacity() const { return capacity_; }
    const TraceConfig& trace() const { return trace_; }
    uint64_t rays() const { return rays_; }
    uint64_t shadow_rays() const { return shadow_rays_; }
    uint32_t waves() const { return waves_; }

private:
    void launch_wave(const WaveHeader& h, bool any_nee, bool two, cudaStream_t st);
    int device_, sm_count_;
    uint32_t capacity_;
    bool use_graphs_;
    TraceConfig trace_;           // grid-form traversal variant of the extend and shadow kernels
    DeviceBuffer paths_;          // path state for `capacity_` slots (+ job, pixel, sample, depth arrays)
    DeviceBuffer desc_;           // header + segments + job table
    void* host_desc_ = nullptr;   // pinned staging of the descriptor
    size_t desc_bytes_ = 0;
    struct GraphSlot {
        uint32_t bounces = 0;
        bool nee = false;
        bool two = false;   // the wave holds a two-level scene
        cudaGraphExec_t exec = nullptr;
    };
    std::vector<GraphSlot> graphs_;
    uint64_t rays_ = 0, shadow_rays_ = 0;
    uint32_t waves_ = 0;
    int blocks_ext_ = 0, blocks_shade_[5] = {0, 0, 0, 0, 0}, blocks_sh_ = 0, blocks_simple_ = 0;
    int blocks_ext_two_ = 0, blocks_sh_two_ = 0;
};

}  // namespace rt
