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
    // this wave: the job's slots are [wave_start, wave_start + take), holding its (sample * W*H + pixel)
    // indices [cursor0, cursor0 + take); finish threads [finish_start, finish_start + min(take, W*H)),
    // one per pixel, sum each pixel's samples of the wave in sample order
    uint64_t cursor0;
    uint32_t wave_start;
    uint32_t take;
    uint32_t finish_start;
    uint32_t pad3;
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
    uint32_t finish_total;   // finish threads (sum over jobs of min(take, W*H))
    uint32_t pad[3];         // 32 bytes: the job table after the segments stays 16-byte aligned
};
static_assert(sizeof(WaveHeader) == 32, "WaveHeader must stay 32 bytes");

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
    bool resolved = false;   // every sample is scheduled (set when the job's last wave is packed)
    void* owner = nullptr;   // the caller's record of the job (the server's request)
};

class BatchEngine {
public:
    // `lanes` path-state buffers (1 to 4) of `wave_capacity` slots each; waves rotate over them so that
    // one wave's last bounces overlap the next waves' first ones.
    BatchEngine(int device, int sm_count, uint32_t wave_capacity, bool use_graphs,
                const TraceConfig& trace = TraceConfig(), int lanes = 1);
    ~BatchEngine();
    BatchEngine(const BatchEngine&) = delete;
    BatchEngine& operator=(const BatchEngine&) = delete;

    // Allocates the job's per-pixel state (24 bytes per pixel); the job must outlive its waves.  With a
    // pool, the allocation is stream-ordered on `st` (DeviceBuffer::alloc_async).
    static void prepare(BatchJob& job, cudaMemPool_t pool = nullptr, cudaStream_t st = nullptr);
    // Waves are packed from `jobs`: an equal share of the capacity per job with samples left, leftovers
    // to the first jobs (or, with `fifo`, each job in list order taking all it can use); a job in the
    // reference's mode places at most one sample of each pixel in a wave, a NEE+MIS job any number (the
    // finish kernel sums each pixel's samples of the wave in sample order).  Wave k runs on lane k mod lanes, on the lane's own stream.  Each
    // wave's finish kernel (the per-pixel sums) runs after the previous wave's, so a pixel's samples are
    // summed in sample order; a wave holding a job whose samples carry state from the pixel's previous
    // sample (the reference's seeding mode) starts only after the previous wave's finish.
    //
    // Packs the next wave into the next lane, which must be free (lane_free()), and launches it.
    // Returns false when no job has samples left to schedule.  `members` and `completed` (optional)
    // receive the jobs in the wave and the jobs whose last samples it holds.
    bool submit_wave(const std::vector<BatchJob*>& jobs, bool fifo, std::vector<BatchJob*>* members = nullptr,
                     std::vector<BatchJob*>* completed = nullptr);
    bool lane_free() const { return !lanes_[submitted_ % lanes_.size()].pending; }
    bool pending() const { return retired_ < submitted_; }
    // Waits for the oldest wave in flight and adds its ray counts; throws on a device error flag.
    void wait_oldest();
    // Waits for every wave in flight without reading their results (error and shutdown paths).
    void drain();
    // The lanes' next work waits for the work queued on `st` so far.
    void order_after(cudaStream_t st);
    // The work queued on `st` from now on waits for every wave submitted so far.
    void order_before(cudaStream_t st);
    // Runs waves until every job is resolved, as many in flight as the engine has lanes.  Ordered
    // after the work queued on `st` before the call; returns with every wave complete and the work
    // queued on `st` afterwards ordered after them.
    void run_all(const std::vector<BatchJob*>& jobs, cudaStream_t st, bool fifo = false);
    uint32_t capacity() const { return capacity_; }
    int lanes() const { return (int)lanes_.size(); }
    const TraceConfig& trace() const { return trace_; }
    uint64_t rays() const { return rays_; }
    uint64_t shadow_rays() const { return shadow_rays_; }
    // traversal work (nodes, triangles of closest and any-hit rays, shaded hits) over the waves collected
    // so far: counted by the cooperative kernels always, and by the grid-form kernels while counting is on
    const RenderStats& work() const { return work_; }
    // Counting on: waves launched from now on run the grid form's counting kernels (default block size and
    // stack depth; the same traversal, so the same images) where they would run the grid form.
    void set_counting(bool on) { count_ = on; }
    uint32_t waves() const { return waves_; }

private:
    struct GraphSlot {
        uint32_t bounces = 0;
        bool nee = false;
        bool two = false;   // the wave holds a two-level scene
        bool count = false; // counting kernels (traversal work)
        cudaGraphExec_t exec = nullptr;
    };
    struct Lane {
        DeviceBuffer paths;             // path state for the capacity's slots (+ job, pixel, sample, depth)
        DeviceBuffer desc;              // header + segments + job table
        void* host_desc = nullptr;      // pinned staging of the descriptor
        uint32_t* host_counters = nullptr;   // pinned copy of the wave's counters
        cudaStream_t stream = nullptr;  // run_all's stream for this lane
        cudaEvent_t finished = nullptr; // after the lane's last finish kernel and resolves
        cudaEvent_t done = nullptr;     // after the lane's last counter copy
        bool pending = false;           // a wave whose counters are not collected yet
        std::vector<GraphSlot> graphs;  // captured wave bodies (pointers into this lane's buffers)
    };
    struct Packed {
        WaveHeader hdr;
        bool any_nee = false, two = false, carries = false;
        std::vector<BatchJob*> members, completed;
    };
    // Packs the next wave into the lane's host descriptor; hdr.count == 0 when nothing is left.
    Packed pack(const std::vector<BatchJob*>& jobs, bool fifo, Lane& L);
    // Descriptor upload + wave body (init and the bounce kernels) on `s`.
    void launch_body(Lane& L, const Packed& pk, cudaStream_t s);
    // Finish kernel, resolves of the completed jobs, counter copy on `s`.
    void launch_finish(Lane& L, const Packed& pk, cudaStream_t s);
    // Adds a synchronized lane's counters to the totals; throws on a device error flag.
    void collect(Lane& L);
    // Waits for and releases every lane's streams, events, graphs and buffers.
    void release_lanes();
    int device_, sm_count_;
    uint32_t capacity_;
    bool use_graphs_;
    TraceConfig trace_;           // grid-form traversal variant of the extend and shadow kernels
    size_t desc_bytes_ = 0;
    std::vector<Lane> lanes_;
    uint64_t rays_ = 0, shadow_rays_ = 0;
    RenderStats work_;
    uint32_t waves_ = 0;
    uint64_t submitted_ = 0, retired_ = 0;   // waves launched / waited for
    int blocks_ext_ = 0, blocks_shade_[5] = {0, 0, 0, 0, 0}, blocks_sh_ = 0, blocks_simple_ = 0;
    int blocks_ext_two_ = 0, blocks_sh_two_ = 0;
    int blocks_ext_cnt_ = 0, blocks_sh_cnt_ = 0, blocks_ext_two_cnt_ = 0, blocks_sh_two_cnt_ = 0;
    bool count_ = false;
};

}  // namespace rt
