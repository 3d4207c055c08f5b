// Render-request server (see server.h).  One loop thread owns every device resource of the server:
// admission, uploads, evictions and the waves all run there; client threads only queue requests, read
// statuses and copy kept images out.
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

namespace rt {

namespace {
constexpr size_t kPixelStateBytes = 24;   // per pixel: carried RNG, accumulatedDistance, sums, count
constexpr size_t kImageBytes = 16;        // per pixel: RGBA32F
constexpr size_t kPathBytes = 164;        // per wave slot of the batch engine
}  // namespace

double Server::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

Server::Server(int device, int sm_count, const ServerConfig& cfg) : device_(device), cfg_(cfg) {
    if (cfg_.max_active == 0 || cfg_.max_active > kMaxWaveSegments / 2)
        fail(REINA_ERR_INVALID, "max_active_jobs must be in 1.." + std::to_string(kMaxWaveSegments / 2));
    const uint32_t wave = cfg_.wave_paths ? cfg_.wave_paths : (uint32_t)REINA_SERVER_WAVE_PATHS;
    const uint32_t lanes = cfg_.lanes ? cfg_.lanes : (uint32_t)REINA_SERVER_WAVE_LANES;
    if (lanes > 16) fail(REINA_ERR_INVALID, "wave_lanes must be in 0..16");
    reserved_ = lanes * (uint64_t)wave * kPathBytes + (64u << 20);   // path state of the lanes + descriptors and slack
    if (cfg_.budget < reserved_)
        fail(REINA_ERR_BUDGET, "memory budget " + std::to_string(cfg_.budget) + " B is below the engine's " +
                                   std::to_string(reserved_) + " B of path state");
    check_cuda(cudaSetDevice(device_), "cudaSetDevice");
    try {
        check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        // requests' pixel state and own images come from this pool, stream-ordered on stream_, so that
        // admitting and finishing requests does not wait for the waves in flight
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device_;
        check_cuda(cudaMemPoolCreate(&pool_, &props), "cudaMemPoolCreate");
        uint64_t keep = cfg_.budget;   // freed memory stays in the pool up to the budget
        check_cuda(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
        TraceConfig trace;
        trace.refill = kDefaultWaveRefill;
        engine_ = std::make_unique<BatchEngine>(device_, sm_count, wave, cfg_.graphs, trace, (int)lanes);
    } catch (...) {   // the destructor does not run for a constructor that throws
        engine_.reset();
        if (pool_) cudaMemPoolDestroy(pool_);
        if (stream_) cudaStreamDestroy(stream_);
        throw;
    }
    t0_ = now();
    thread_ = std::thread([this] { loop(); });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    if (thread_.joinable()) thread_.join();
    cudaSetDevice(device_);
    {
        std::lock_guard<std::mutex> lk(mu_);
        for (Request* r : running_) finish(*r, kReqCancelled, 0, "server destroyed");
        for (Request* r : queue_) finish(*r, kReqCancelled, 0, "server destroyed");
        running_.clear();
        queue_.clear();
    }
    cv_done_.notify_all();
    requests_.clear();
    images_.clear();
    engine_.reset();
    if (stream_) cudaStreamSynchronize(stream_);
    if (pool_) cudaMemPoolDestroy(pool_);
    if (stream_) cudaStreamDestroy(stream_);
}

uint32_t Server::add_scene(Scene* scene) {
    if (!scene || !scene->built()) fail(REINA_ERR_STATE, "scene is not built");
    if (scene->device() != device_) fail(REINA_ERR_INVALID, "scene belongs to another device");
    std::lock_guard<std::mutex> lk(mu_);
    SceneSlot s;
    s.scene = scene;
    s.last_use = ++tick_;
    if (scene->resident()) {
        const size_t b = scene->upload_bytes();
        if (resident_ + b + reserved_ <= cfg_.budget) {
            resident_ += b;
            peak_ = std::max(peak_, resident_);
        } else {
            check_cuda(cudaSetDevice(device_), "cudaSetDevice");
            scene->release_device();
        }
    }
    scenes_.push_back(s);
    return (uint32_t)(scenes_.size() - 1);
}

size_t Server::request_bytes(const RequestSpec& s) const {
    const size_t px = (size_t)s.opt.width * s.opt.height;
    return px * (kPixelStateBytes + kImageBytes);
}

uint64_t Server::submit(const RequestSpec& spec) {
    if (spec.opt.megakernel) fail(REINA_ERR_INVALID, "served requests run the wavefront (options.flags must be 0)");
    if (!spec.host_out && spec.image_key == 0) fail(REINA_ERR_INVALID, "a request needs a host image or an image key");
    std::lock_guard<std::mutex> lk(mu_);
    if (stop_) fail(REINA_ERR_STATE, "server is shutting down");
    if (spec.scene >= scenes_.size()) fail(REINA_ERR_INVALID, "unknown server scene id");
    const Scene& sc = *scenes_[spec.scene].scene;
    if (spec.opt.mode == kModeNeeMis && sc.emissive_data().size() > 0 && !(spec.pc.totalEmissiveWeight > 0.0f))
        fail(REINA_ERR_INVALID, "totalEmissiveWeight must be positive for NEE");
    const uint64_t need = request_bytes(spec) + sc.upload_bytes();
    if (need + reserved_ > cfg_.budget)
        fail(REINA_ERR_BUDGET, "request needs " + std::to_string(need) + " B of device memory; the budget leaves " +
                                   std::to_string(cfg_.budget - reserved_) + " B");
    auto r = std::make_unique<Request>();
    r->id = next_id_++;
    r->spec = spec;
    r->t_submit = now();
    if (first_submit_ < 0) first_submit_ = r->t_submit;
    Request* p = r.get();
    requests_.emplace(p->id, std::move(r));
    queue_.push_back(p);
    counters_.submitted++;
    cv_work_.notify_one();
    return p->id;
}

RequestStatus Server::poll(uint64_t id) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) fail(REINA_ERR_INVALID, "unknown request id");
    return it->second->status;
}

RequestStatus Server::wait(uint64_t id, double timeout_s) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) fail(REINA_ERR_INVALID, "unknown request id");
    Request* r = it->second.get();
    auto done = [&] { return r->status.state >= kReqDone; };
    if (timeout_s < 0) cv_done_.wait(lk, done);
    else cv_done_.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
    return r->status;
}

void Server::cancel(uint64_t id) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) fail(REINA_ERR_INVALID, "unknown request id");
    it->second->cancel = true;
    cv_work_.notify_one();
}

void Server::fetch_image(uint64_t key, float* host_out, uint32_t* w, uint32_t* h) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = images_.find(key);
    if (it == images_.end() || !it->second.valid) fail(REINA_ERR_STATE, "no finished image under this key");
    ImageSlot& im = it->second;
    if (im.busy) fail(REINA_ERR_STATE, "a running request is writing this image");
    if (w) *w = im.w;
    if (h) *h = im.h;
    if (!host_out) return;
    const size_t bytes = (size_t)im.w * im.h * kImageBytes;
    if (im.dev.get()) {
        check_cuda(cudaSetDevice(device_), "cudaSetDevice");
        check_cuda(cudaMemcpy(host_out, im.dev.get(), bytes, cudaMemcpyDeviceToHost), "D2H image");
    } else {
        std::memcpy(host_out, im.host.data(), bytes);
    }
}

ServerStats Server::stats() {
    std::lock_guard<std::mutex> lk(mu_);
    ServerStats s = counters_;
    s.queued = queue_.size();
    s.running = running_.size();
    std::vector<double> l = latencies_;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        const size_t k = (size_t)std::min<double>((double)l.size() - 1, std::ceil(q * (double)l.size()) - 1);
        return l[k];
    };
    s.p50 = pct(0.50);
    s.p99 = pct(0.99);
    double sum = 0;
    for (double x : l) sum += x;
    s.mean = l.empty() ? 0.0 : sum / (double)l.size();
    s.max = l.empty() ? 0.0 : l.back();
    s.uptime_s = now() - t0_;
    s.first_submit_to_last_done_s = first_submit_ < 0 ? 0.0 : std::max(0.0, last_done_ - first_submit_);
    s.resident_bytes = resident_;
    s.peak_resident_bytes = peak_;
    s.budget_bytes = cfg_.budget;
    s.reserved_bytes = reserved_;
    return s;
}

// Evicts least-recently-used idle scenes and kept images (never those `r` needs) until `need` more bytes
// fit the budget.  Returns false if they cannot.
bool Server::make_room(size_t need, const Request& r) {
    while (resident_ + need + reserved_ > cfg_.budget) {
        uint64_t best = UINT64_MAX;
        SceneSlot* bs = nullptr;
        ImageSlot* bi = nullptr;
        for (size_t k = 0; k < scenes_.size(); ++k) {
            SceneSlot& s = scenes_[k];
            if (k != r.spec.scene && s.active == 0 && s.scene->resident() && s.last_use < best) {
                best = s.last_use;
                bs = &s;
                bi = nullptr;
            }
        }
        for (auto& [key, im] : images_) {
            if (key != r.spec.image_key && !im.busy && im.dev.get() && im.last_use < best) {
                best = im.last_use;
                bi = &im;
                bs = nullptr;
            }
        }
        if (bs) {
            resident_ -= bs->scene->upload_bytes();
            bs->scene->release_device();
            counters_.scene_evictions++;
        } else if (bi) {
            const size_t bytes = (size_t)bi->w * bi->h * kImageBytes;
            bi->host.resize((size_t)bi->w * bi->h * 4);
            check_cuda(cudaMemcpy(bi->host.data(), bi->dev.get(), bytes, cudaMemcpyDeviceToHost), "D2H evicted image");
            bi->dev.release();
            resident_ -= bytes;
            counters_.image_evictions++;
        } else {
            return false;
        }
    }
    return true;
}

bool Server::try_admit(Request& r) {
    const RequestSpec& s = r.spec;
    SceneSlot& sc = scenes_[s.scene];
    const size_t px = (size_t)s.opt.width * s.opt.height;
    size_t need = px * kPixelStateBytes;
    ImageSlot* img = nullptr;
    bool fresh_image = false;
    if (s.image_key) {
        auto it = images_.find(s.image_key);
        if (it != images_.end()) {
            img = &it->second;
            if (img->busy) return false;   // the previous request on this key is still running
            const bool same = img->w == s.opt.width && img->h == s.opt.height;
            if (s.pc.sampleBatch > 0 && (!img->valid || !same))
                fail(REINA_ERR_STATE, "progressive request: no finished image of this size under the key");
            if (!same) {
                if (img->dev.get()) resident_ -= (size_t)img->w * img->h * kImageBytes;
                images_.erase(it);
                img = nullptr;
            }
        } else if (s.pc.sampleBatch > 0) {
            fail(REINA_ERR_STATE, "progressive request: no finished image under the key");
        }
        if (!img) fresh_image = true;
        if (!img || !img->dev.get()) need += px * kImageBytes;
    } else {
        need += px * kImageBytes;
    }
    if (!sc.scene->resident()) need += sc.scene->upload_bytes();
    if (!make_room(need, r)) return false;

    if (!sc.scene->resident()) {
        sc.scene->upload();
        resident_ += sc.scene->upload_bytes();
        counters_.scene_uploads++;
    }
    float* d_accum = nullptr;
    try {
        if (s.image_key) {
            if (fresh_image) {
                img = &images_[s.image_key];
                img->w = s.opt.width;
                img->h = s.opt.height;
            }
            if (!img->dev.get()) {
                img->dev.alloc(px * kImageBytes);
                resident_ += px * kImageBytes;
                if (!img->host.empty()) {
                    check_cuda(cudaMemcpy(img->dev.get(), img->host.data(), px * kImageBytes, cudaMemcpyHostToDevice),
                               "H2D restored image");
                    img->host.clear();
                    img->host.shrink_to_fit();
                    counters_.image_restores++;
                }
            }
            d_accum = img->dev.as<float>();
        } else {
            r.accum.alloc_async(px * kImageBytes, pool_, stream_);
            resident_ += px * kImageBytes;
            if (s.pc.sampleBatch > 0)
                check_cuda(cudaMemcpyAsync(r.accum.get(), s.host_out, px * kImageBytes, cudaMemcpyHostToDevice,
                                           stream_), "H2D previous image");
            d_accum = r.accum.as<float>();
        }
        r.job.scene = sc.scene->device_view();
        r.job.pc = s.pc;
        r.job.opt = s.opt;
        r.job.d_accum = d_accum;
        r.job.d_samples = nullptr;
        r.job.owner = &r;
        BatchEngine::prepare(r.job, pool_, stream_);
        // the allocations (and the previous image) are complete before any lane uses them
        check_cuda(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    } catch (...) {
        if (r.accum.get()) {
            resident_ -= px * kImageBytes;
            r.accum.release();
        }
        throw;
    }
    if (img) img->busy = true;
    resident_ += px * kPixelStateBytes;
    r.job_bytes = px * kPixelStateBytes + (s.image_key ? 0 : px * kImageBytes);
    peak_ = std::max(peak_, resident_);
    sc.active++;
    sc.last_use = ++tick_;
    r.t_admit = now();
    r.status.state = kReqRunning;
    r.status.queue_s = r.t_admit - r.t_submit;
    return true;
}

// Releases what a request holds (if it was admitted) and records its final state.
void Server::finish(Request& r, uint32_t state, int error, const std::string& msg) {
    if (r.status.state == kReqRunning) {
        SceneSlot& sc = scenes_[r.spec.scene];
        sc.active--;
        sc.last_use = ++tick_;
        if (r.spec.image_key) {
            auto it = images_.find(r.spec.image_key);
            if (it != images_.end()) {
                it->second.busy = false;
                it->second.last_use = ++tick_;
                if (state == kReqDone) it->second.valid = true;   // the image is written only at completion
            }
        }
        r.job.pixel_state.release();
        r.accum.release();
        resident_ -= r.job_bytes;
    }
    const double t = now();
    r.status.state = state;
    r.status.error = error;
    r.status.message = msg;
    r.status.latency_s = t - r.t_submit;
    if (state == kReqDone) {
        counters_.completed++;
        latencies_.push_back(r.status.latency_s);
        last_done_ = t;
    } else if (state == kReqFailed) {
        counters_.failed++;
    } else {
        counters_.cancelled++;
    }
}

// The loop keeps up to one wave per engine lane in flight: while one runs its last bounces the next are
// already packed and running.  Between steps it drops cancelled requests that no wave in flight
// holds, admits queued requests, and then either launches a wave on a free lane or waits for the oldest
// wave; a request completes when the wave holding its last samples is done.
void Server::loop() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    std::deque<std::vector<Request*>> waves;   // the requests in each wave in flight, oldest first
    double busy_from = 0;
    auto schedulable = [&](const Request* r) { return !r->cancel && r->job.cursor < r->job.total; };
    for (;;) {
        if (!engine_->pending())
            cv_work_.wait(lk, [&] {
                if (stop_ || !queue_.empty()) return true;
                for (const Request* r : running_)
                    if (schedulable(r) || (r->cancel && r->inflight == 0)) return true;
                return false;
            });
        if (stop_) {
            lk.unlock();
            engine_->drain();
            return;
        }
        for (auto it = running_.begin(); it != running_.end();) {
            if ((*it)->cancel && (*it)->inflight == 0) {
                finish(**it, kReqCancelled, 0, "cancelled");
                it = running_.erase(it);
            } else {
                ++it;
            }
        }
        while (!queue_.empty() && running_.size() < cfg_.max_active) {
            Request* r = queue_.front();
            if (r->cancel) {
                queue_.pop_front();
                finish(*r, kReqCancelled, 0, "cancelled");
                continue;
            }
            bool ok = false;
            try {
                ok = try_admit(*r);
            } catch (const Error& e) {
                queue_.pop_front();
                finish(*r, kReqFailed, e.code, e.what());
                continue;
            }
            if (!ok) {
                if (running_.empty()) {   // nothing to wait for: everything evictable was tried
                    queue_.pop_front();
                    finish(*r, kReqFailed, REINA_ERR_BUDGET, "request does not fit the memory budget");
                    continue;
                }
                break;
            }
            queue_.pop_front();
            running_.push_back(r);
        }
        cv_done_.notify_all();
        std::vector<BatchJob*> jobs;
        for (Request* r : running_)
            if (schedulable(r)) jobs.push_back(&r->job);
        if (cfg_.shortest && cfg_.aging > 0.0) {
            // estimated remaining time minus aging x waiting time; stable: ties keep arrival order
            // samples per second: completed samples over the time since the first submission (a
            // nominal 4e8 until the first request completes)
            const double t = now();
            const double rate = samples_done_ > 0.0 && t > first_submit_ ? samples_done_ / (t - first_submit_) : 4e8;
            std::vector<std::pair<double, BatchJob*>> keyed;
            keyed.reserve(jobs.size());
            for (BatchJob* j : jobs) {
                const Request* r = static_cast<const Request*>(j->owner);
                keyed.emplace_back((double)(j->total - j->cursor) / rate - cfg_.aging * (t - r->t_submit), j);
            }
            std::stable_sort(keyed.begin(), keyed.end(),
                             [](const auto& a, const auto& b) { return a.first < b.first; });
            for (size_t k = 0; k < jobs.size(); ++k) jobs[k] = keyed[k].second;
        } else if (cfg_.shortest) {   // fewest samples left first; stable: ties keep arrival order
            std::stable_sort(jobs.begin(), jobs.end(), [](const BatchJob* a, const BatchJob* b) {
                return a->total - a->cursor < b->total - b->cursor;
            });
        }
        const bool launch = !jobs.empty() && engine_->lane_free();
        if (!launch && !engine_->pending()) continue;
        lk.unlock();
        int code = 0;
        std::string err;
        std::vector<BatchJob*> members;
        std::vector<Request*> done;
        bool retired = false;
        try {
            if (launch) {
                if (!engine_->pending()) busy_from = now();
                engine_->submit_wave(jobs, cfg_.fifo || cfg_.shortest, &members);
            } else {
                engine_->wait_oldest();
                retired = true;
            }
        } catch (const Error& e) {
            code = e.code;
            err = e.what();
            engine_->drain();
        }
        if (!code && retired) {
            // the oldest wave is done: requests whose last samples it held are complete; their images go
            // to the host outside the lock (the loop thread alone touches running requests' jobs)
            for (Request* r : waves.front())
                if (--r->inflight == 0 && r->job.resolved && !r->cancel) done.push_back(r);
            waves.pop_front();
            for (Request* r : done)
                if (r->spec.host_out) {
                    const size_t bytes = (size_t)r->spec.opt.width * r->spec.opt.height * kImageBytes;
                    const cudaError_t ce = cudaMemcpy(r->spec.host_out, r->job.d_accum, bytes, cudaMemcpyDeviceToHost);
                    if (ce != cudaSuccess) {
                        code = REINA_ERR_CUDA;
                        err = std::string("D2H result: ") + cudaGetErrorString(ce);
                        engine_->drain();
                        break;
                    }
                }
        }
        lk.lock();
        if (!code && launch) {
            std::vector<Request*> in_wave;
            for (BatchJob* j : members) {
                Request* r = static_cast<Request*>(j->owner);
                r->inflight++;
                in_wave.push_back(r);
            }
            waves.push_back(std::move(in_wave));
        }
        if (!engine_->pending()) counters_.busy_s += now() - busy_from;
        counters_.rays = engine_->rays();
        counters_.shadow_rays = engine_->shadow_rays();
        counters_.waves = engine_->waves();
        if (code) {
            for (Request* r : running_) {
                r->inflight = 0;
                finish(*r, kReqFailed, code, err);
            }
            running_.clear();
            waves.clear();
        } else {
            for (Request* r : done) {
                samples_done_ += (double)r->job.total;
                finish(*r, kReqDone, 0, "");
                running_.erase(std::find(running_.begin(), running_.end(), r));
            }
        }
        cv_done_.notify_all();
    }
}

}  // namespace rt
