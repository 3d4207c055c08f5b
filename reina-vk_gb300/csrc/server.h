// Render-request server: a loop thread that admits requests as they arrive, by device-memory budget,
// keeps scenes and kept accumulation images resident with least-recently-used eviction, and runs all
// admitted requests together in the waves of a BatchEngine (continuous batching: requests join and
// leave between waves).
#pragma once

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime_api.h>

#include "batch.h"
#include "scene.h"

namespace rt {

enum RequestState : uint32_t { kReqQueued = 0, kReqRunning = 1, kReqDone = 2, kReqFailed = 3, kReqCancelled = 4 };

struct ServerConfig {
    uint64_t budget = 0;          // device bytes for scenes, images, requests and the engine's path state
    uint32_t max_active = 512;    // requests sharing the waves
    uint32_t wave_paths = 0;
    uint32_t lanes = 0;           // waves in flight (0 = REINA_SERVER_WAVE_LANES)
    bool graphs = true;
    bool fifo = false;            // wave slots to the oldest requests first (default: fair share)
    bool shortest = false;        // wave slots to the requests with the fewest samples left first
    double aging = 0.0;           // shortest: seconds of priority per second since submission
};

struct RequestSpec {
    uint32_t scene = 0;           // server scene id
    uint64_t image_key = 0;       // 0: none; else the accumulation image stays resident under this key
    RtPushConsts pc{};
    RenderOpts opt;
    float* host_out = nullptr;    // W*H RGBA32F, written at completion (may be null with an image key)
};

struct RequestStatus {
    uint32_t state = kReqQueued;
    int error = 0;
    double latency_s = 0, queue_s = 0;
    std::string message;
};

struct ServerStats {
    uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, queued = 0, running = 0;
    double p50 = 0, p99 = 0, mean = 0, max = 0;    // latency (submit -> result on the host) of completed requests
    double uptime_s = 0, busy_s = 0;               // since creation; wall time inside waves
    double first_submit_to_last_done_s = 0;
    uint64_t rays = 0, shadow_rays = 0, waves = 0;
    uint64_t scene_uploads = 0, scene_evictions = 0, image_evictions = 0, image_restores = 0;
    uint64_t resident_bytes = 0, peak_resident_bytes = 0, budget_bytes = 0, reserved_bytes = 0;
};

class Server {
public:
    Server(int device, int sm_count, const ServerConfig& cfg);
    ~Server();   // cancels queued and running requests and joins the loop
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    // The scene must be built for this server's device and outlive the server; it is released from the
    // device now and uploaded again when a request needs it.
    uint32_t add_scene(Scene* scene);
    uint64_t submit(const RequestSpec& spec);        // throws Error(REINA_ERR_BUDGET) if it can never fit
    RequestStatus poll(uint64_t id);
    RequestStatus wait(uint64_t id, double timeout_s);
    void cancel(uint64_t id);
    void fetch_image(uint64_t key, float* host_out, uint32_t* w, uint32_t* h);
    ServerStats stats();

private:
    struct SceneSlot {
        Scene* scene = nullptr;
        uint64_t last_use = 0;
        uint32_t active = 0;      // running requests using it
    };
    struct ImageSlot {
        DeviceBuffer dev;         // resident copy
        std::vector<float> host;  // evicted copy
        uint32_t w = 0, h = 0;
        uint64_t last_use = 0;
        bool busy = false;        // a running request writes it
        bool valid = false;       // holds a finished image
    };
    struct Request {
        uint64_t id = 0;
        RequestSpec spec;
        RequestStatus status;
        double t_submit = 0, t_admit = 0;
        bool cancel = false;
        uint32_t inflight = 0;    // waves in flight holding samples of this request
        size_t job_bytes = 0;     // accounted while running
        BatchJob job;
        DeviceBuffer accum;       // own accumulation image when there is no image key
    };

    void loop();
    bool try_admit(Request& r);               // loop thread, under the lock
    bool make_room(size_t need, const Request& r);
    void finish(Request& r, uint32_t state, int error, const std::string& msg);
    double now() const;
    size_t request_bytes(const RequestSpec& s) const;

    int device_;
    ServerConfig cfg_;
    cudaStream_t stream_ = nullptr;   // orders the pool's allocations and frees
    cudaMemPool_t pool_ = nullptr;    // requests' pixel state and own images
    std::unique_ptr<BatchEngine> engine_;
    std::thread thread_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    bool stop_ = false;
    uint64_t next_id_ = 1, tick_ = 0;
    std::vector<SceneSlot> scenes_;
    std::unordered_map<uint64_t, ImageSlot> images_;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> requests_;
    std::deque<Request*> queue_;
    std::vector<Request*> running_;
    uint64_t resident_ = 0, peak_ = 0, reserved_ = 0;
    std::vector<double> latencies_;
    ServerStats counters_;
    double t0_ = 0, first_submit_ = -1, last_done_ = 0;
    double samples_done_ = 0;     // samples of completed requests (the aging key's rate estimate)
};

}  // namespace rt
