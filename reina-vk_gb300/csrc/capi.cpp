// C ABI of the library (include/reina/reina_c.h): handles, status codes and thread-local messages.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <unordered_set>
#include <vector>

#include <cuda_runtime_api.h>

#include "../../include/reina/reina_c.h"
#include "autotune.h"
#include "batch.h"
#include "config.h"
#include "errors.h"
#include "generators.h"
#include "image.h"
#include "kat.h"
#include "kernels.h"
#include "loaders.h"
#include "post.h"
#include "render.h"
#include "scene.h"
#include "server.h"

using rt::check_cuda;
using rt::fail;

struct reina_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t streams[2] = {nullptr, nullptr};
    rt::DeviceBuffer err;        // u32 device error flag, OR-ed by kernels
    rt::DeviceBuffer counters;   // u64 x 2 traversal counters
    rt::DeviceBuffer fetch;      // ring of u32 ray-fetch counters, one per ray-cast launch in flight
    std::atomic<uint32_t> fetch_slot{0};
    uint32_t* err_host = nullptr;   // page-locked ring of words the error flag is read back into
    std::atomic<uint32_t> err_slot{0};
    ~reina_ctx() {
        if (err_host) cudaFreeHost(err_host);
    }
    rt::TraceConfig trace;       // ray-cast traversal launch configuration (reina_tuning)
    rt::TraceConfig wave_trace = wave_default();   // the wavefront kernels' (reina_tuning.wave_refill)
    static rt::TraceConfig wave_default() {
        rt::TraceConfig c;
        c.refill = rt::kDefaultWaveRefill;
        return c;
    }
    uint32_t* next_fetch_counter() { return fetch.as<uint32_t>() + (fetch_slot.fetch_add(1) % kFetchSlots); }
    static constexpr uint32_t kFetchSlots = 256;
    rt::DeviceBuffer rays, hits; // staging for host-buffer ray casts
    rt::RenderWorkspace render;  // wavefront path state and queues
    rt::DeviceBuffer accum, samples;   // staging for host-buffer renders
    rt::PostWorkspace post;      // bloom intermediate images
    rt::DeviceBuffer rgba8, combined;  // staging for host-buffer post-processing
    uint32_t wave_paths = REINA_DEFAULT_WAVE_PATHS;
    uint32_t batch_flags = 0;
    uint32_t wave_lanes = REINA_DEFAULT_WAVE_LANES;   // waves in flight in the batch engine
    std::unique_ptr<rt::BatchEngine> batch;   // built on the first batched render
    rt::TuneCache tune;          // autotuned configurations
    uint32_t autotune_mode = REINA_AUTOTUNE_OFF;
    std::mutex scenes_mu;
    std::unordered_set<reina_scene*> scenes;  // live scenes; detached (device memory freed) on destroy
    std::unordered_set<reina_server*> servers;   // destroyed before the context
};

struct reina_scene {
    reina_ctx* ctx = nullptr;
    std::unique_ptr<rt::Scene> s;
};

struct reina_server {
    reina_ctx* ctx = nullptr;
    std::unique_ptr<rt::Server> srv;
    std::vector<reina_scene*> scenes;   // owned
};

namespace {

thread_local std::string g_error;

template <class F>
int guard(F&& f) {
    try {
        f();
        return REINA_OK;
    } catch (const rt::Error& e) {
        g_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_error = "host allocation failed";
        return REINA_ERR_OOM;
    } catch (const std::exception& e) {
        g_error = e.what();
        return REINA_ERR_INVALID;
    } catch (...) {
        g_error = "unknown error";
        return REINA_ERR_INVALID;
    }
}

void need(bool cond, const char* msg) {
    if (!cond) fail(REINA_ERR_INVALID, msg);
}

void use_device(const reina_ctx* ctx) {
    if (ctx->device < 0) fail(REINA_ERR_STATE, "host-only context (device -1) cannot run GPU work");
    check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
}

const rt::Scene& built_scene(const reina_scene* scene) {
    need(scene != nullptr, "scene is NULL");
    if (!scene->ctx) fail(REINA_ERR_STATE, "the scene's context has been destroyed");
    if (!scene->s->built()) fail(REINA_ERR_STATE, "scene is not built (call reina_scene_build)");
    if (scene->ctx->device >= 0 && !scene->s->resident()) fail(REINA_ERR_STATE, "scene is not resident on the GPU");
    return *scene->s;
}

rt::ModelData to_model(const reina_model_data* m) {
    need(m != nullptr, "model data is NULL");
    need(m->vertices || m->vertex_count == 0, "vertices is NULL");
    need(m->indices || m->index_count == 0, "indices is NULL");
    need(m->tbns || m->tbn_count == 0, "tbns is NULL");
    need(m->tbn_indices || m->tbn_index_count == 0, "tbn_indices is NULL");
    need(m->tex_coords || m->tex_coord_count == 0, "tex_coords is NULL");
    need(m->tex_indices || m->tex_index_count == 0, "tex_indices is NULL");
    rt::ModelData d;
    d.vertices.assign(m->vertices, m->vertices + 4 * m->vertex_count);
    d.indices.assign(m->indices, m->indices + m->index_count);
    d.tbns.assign(m->tbns, m->tbns + 9 * m->tbn_count);
    d.tbn_indices.assign(m->tbn_indices, m->tbn_indices + m->tbn_index_count);
    d.tex_coords.assign(m->tex_coords, m->tex_coords + 2 * m->tex_coord_count);
    d.tex_indices.assign(m->tex_indices, m->tex_indices + m->tex_index_count);
    return d;
}

uint32_t check_device_errors(reina_ctx* ctx, cudaStream_t st) {
    // read back into a page-locked word (a pageable destination would stage the copy): one word of the
    // ring per call, so that calls on other streams do not share it
    uint32_t* w = ctx->err_host + (ctx->err_slot.fetch_add(1) % reina_ctx::kFetchSlots);
    check_cuda(cudaMemcpyAsync(w, ctx->err.get(), sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync err");
    check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    const uint32_t e = *w;
    if (e) {
        check_cuda(cudaMemsetAsync(ctx->err.get(), 0, sizeof(uint32_t), st), "cudaMemsetAsync err");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    }
    return e;
}

// Device address of a page-locked host buffer mapped for `device` (16-byte aligned), or NULL for any other
// memory (pageable, device memory, or pinned for another device).
const void* host_device_pointer(const void* p, int device) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();   // clear the error of an unknown pointer
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || a.device != device || !a.devicePointer || ((uintptr_t)a.devicePointer % 16) != 0)
        return nullptr;
    return a.devicePointer;
}
void* host_device_pointer(void* p, int device) {
    return const_cast<void*>(host_device_pointer(static_cast<const void*>(p), device));
}

// The traversal configuration for a workload: the cached autotuned one when the context uses the
// cache and has an entry, else the context's tuning.
rt::TraceConfig trace_for(const reina_ctx* ctx, uint32_t kind, uint64_t triangles, uint64_t size) {
    rt::TuneEntry e;
    if (ctx->autotune_mode == REINA_AUTOTUNE_CACHED &&
        ctx->tune.get(kind, rt::tune_bucket(triangles), rt::tune_bucket(size), &e))
        return e.trace;
    return kind == rt::kTuneRender || kind == rt::kTuneBatch ? ctx->wave_trace : ctx->trace;
}

// reina_tuning's refill fields <-> TraceConfig::refill (0 = grid form).
int refill_from_abi(uint32_t v, int dflt) { return v == 0 ? dflt : (v == REINA_REFILL_GRID ? 0 : (int)v); }
uint32_t refill_to_abi(int r) { return r == 0 ? (uint32_t)REINA_REFILL_GRID : (uint32_t)r; }

}  // namespace

extern "C" {

const char* reina_last_error(void) { return g_error.c_str(); }

const char* reina_version(void) { return "reina-gb300 0.1 sm_103a"; }

int reina_ctx_create(const reina_ctx_options* options, reina_ctx** out_ctx) {
    return guard([&] {
        need(out_ctx != nullptr, "out_ctx is NULL");
        *out_ctx = nullptr;
        auto ctx = std::make_unique<reina_ctx>();
        ctx->device = options ? options->device : 0;
        if (ctx->device == -1) {   // host-only: scene assembly and BVH build without a GPU
            *out_ctx = ctx.release();
            return;
        }
        int count = 0;
        check_cuda(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
        if (ctx->device < 0 || ctx->device >= count) fail(REINA_ERR_INVALID, "device ordinal out of range");
        use_device(ctx.get());
        check_cuda(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device), "cudaDeviceGetAttribute");
        for (auto& s : ctx->streams) check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
        // ray casts take their ordering scratch from the device's default stream-ordered pool: keep freed
        // blocks in the pool instead of returning them at every synchronization
        cudaMemPool_t pool;
        check_cuda(cudaDeviceGetDefaultMemPool(&pool, ctx->device), "cudaDeviceGetDefaultMemPool");
        uint64_t keep = 1ull << 30;
        check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
        ctx->err.alloc(sizeof(uint32_t));
        ctx->counters.alloc(2 * sizeof(unsigned long long));
        ctx->fetch.alloc(reina_ctx::kFetchSlots * sizeof(uint32_t));
        check_cuda(cudaMallocHost(reinterpret_cast<void**>(&ctx->err_host), reina_ctx::kFetchSlots * sizeof(uint32_t)),
                   "cudaMallocHost");
        check_cuda(cudaMemset(ctx->err.get(), 0, sizeof(uint32_t)), "cudaMemset");
        *out_ctx = ctx.release();
    });
}

void reina_ctx_destroy(reina_ctx* ctx) {
    if (!ctx) return;
    while (!ctx->servers.empty()) reina_server_destroy(*ctx->servers.begin());
    if (ctx->device >= 0) cudaSetDevice(ctx->device);
    {
        // scenes outliving their context keep only their handle: free their device memory now
        std::lock_guard<std::mutex> lock(ctx->scenes_mu);
        for (reina_scene* sc : ctx->scenes) {
            sc->s.reset();
            sc->ctx = nullptr;
        }
        ctx->scenes.clear();
    }
    for (auto& s : ctx->streams)
        if (s) cudaStreamDestroy(s);
    delete ctx;
}

int reina_ctx_sm_count(const reina_ctx* ctx) { return ctx ? ctx->sm_count : 0; }

int reina_ctx_set_tuning(reina_ctx* ctx, const reina_tuning* t) {
    return guard([&] {
        need(ctx && t, "NULL argument");
        need(t->refill <= 32 || t->refill == REINA_REFILL_GRID, "refill must be in 0..32 or REINA_REFILL_GRID");
        need(t->wave_refill <= 32 || t->wave_refill == REINA_REFILL_GRID,
             "wave_refill must be in 0..32 or REINA_REFILL_GRID");
        need((t->batch_flags & ~(uint32_t)(REINA_BATCH_NO_GRAPHS | REINA_BATCH_FAIR_SHARE)) == 0, "unknown batch flags");
        need(t->wave_lanes <= 16, "wave_lanes must be in 0..16");
        const uint32_t lanes = t->wave_lanes ? t->wave_lanes : (uint32_t)REINA_DEFAULT_WAVE_LANES;
        const uint32_t wave = t->wave_paths ? t->wave_paths : (uint32_t)REINA_DEFAULT_WAVE_PATHS;
        need(wave <= (1u << 26), "wave_paths must be at most 2^26");
        rt::TraceConfig tc;
        tc.refill = refill_from_abi(t->refill, rt::kDefaultRefill);
        tc.block = (int)(t->trace_block ? t->trace_block : rt::kTraceBlock);
        tc.stack = (int)(t->trace_stack ? t->trace_stack : rt::kDefaultTraceStack);
        need(t->trace_order <= REINA_ORDER_COHERENT, "trace_order must be REINA_ORDER_INPUT or REINA_ORDER_COHERENT");
        tc.sort = t->trace_order == REINA_ORDER_COHERENT ? 1 : 0;
        need(rt::valid_trace_config(tc), "trace_block must be 64, 128 or 256 and trace_stack 8, 12 or 16");
        rt::TraceConfig wc = tc;
        wc.refill = refill_from_abi(t->wave_refill, rt::kDefaultWaveRefill);
        wc.sort = 0;
        const bool engine_changed = wc.block != ctx->wave_trace.block || wc.stack != ctx->wave_trace.stack ||
                                    wc.refill != ctx->wave_trace.refill;
        ctx->trace = tc;
        ctx->wave_trace = wc;
        if (wave != ctx->wave_paths || t->batch_flags != ctx->batch_flags || lanes != ctx->wave_lanes || engine_changed) {
            if (ctx->batch && ctx->device >= 0) check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice");
            ctx->batch.reset();
            ctx->wave_paths = wave;
            ctx->batch_flags = t->batch_flags;
            ctx->wave_lanes = lanes;
        }
    });
}

int reina_ctx_get_tuning(const reina_ctx* ctx, reina_tuning* out) {
    return guard([&] {
        need(ctx && out, "NULL argument");
        std::memset(out, 0, sizeof(*out));
        out->refill = refill_to_abi(ctx->trace.refill);
        out->wave_refill = refill_to_abi(ctx->wave_trace.refill);
        out->trace_block = (uint32_t)ctx->trace.block;
        out->trace_stack = (uint32_t)ctx->trace.stack;
        out->trace_order = ctx->trace.sort ? REINA_ORDER_COHERENT : REINA_ORDER_INPUT;
        out->wave_paths = ctx->wave_paths;
        out->batch_flags = ctx->batch_flags;
        out->wave_lanes = ctx->wave_lanes;
    });
}

int reina_scene_create(reina_ctx* ctx, reina_scene** out_scene) {
    return guard([&] {
        need(ctx && out_scene, "NULL argument");
        auto s = std::make_unique<reina_scene>();
        s->ctx = ctx;
        s->s = std::make_unique<rt::Scene>(ctx->device);
        std::lock_guard<std::mutex> lock(ctx->scenes_mu);
        ctx->scenes.insert(s.get());
        *out_scene = s.release();
    });
}

void reina_scene_destroy(reina_scene* scene) {
    if (!scene) return;
    if (reina_ctx* ctx = scene->ctx) {
        {
            std::lock_guard<std::mutex> lock(ctx->scenes_mu);
            ctx->scenes.erase(scene);
        }
        if (ctx->device >= 0) cudaSetDevice(ctx->device);
    }
    delete scene;
}

int reina_scene_define_object(reina_scene* scene, const reina_model_data* model, uint32_t* out_object_id) {
    return guard([&] {
        need(scene && scene->s && out_object_id, "NULL argument");
        *out_object_id = scene->s->define_object(to_model(model));
    });
}

int reina_scene_add_instance(reina_scene* scene, uint32_t object_id, const float transform[16],
                             const reina_material* material) {
    return guard([&] {
        need(scene && scene->s && transform && material, "NULL argument");
        scene->s->add_instance(object_id, transform, *material);
    });
}

int reina_scene_add_instance_per_face(reina_scene* scene, uint32_t object_id, const float transform[16],
                                      const reina_material* materials, uint32_t material_count,
                                      const uint32_t* face_material) {
    return guard([&] {
        need(scene && scene->s && transform, "NULL argument");
        scene->s->add_instance_per_face(object_id, transform, materials, material_count, face_material);
    });
}

int reina_scene_build(reina_scene* scene, uint32_t require_emissive) {
    return guard([&] {
        need(scene && scene->s, "scene is NULL");
        if (scene->ctx->device >= 0) use_device(scene->ctx);
        scene->s->build(require_emissive != 0);
    });
}

float reina_scene_emissive_weight(const reina_scene* scene) {
    return (scene && scene->s) ? scene->s->emissive_weight() : 0.0f;
}

int reina_scene_get_stats(const reina_scene* scene, reina_scene_stats* out) {
    return guard([&] {
        const rt::Scene& s = built_scene(scene);
        need(out != nullptr, "out_stats is NULL");
        std::memset(out, 0, sizeof(*out));
        out->triangle_count = s.triangle_count();
        out->instance_count = s.instance_count();
        out->node_count = s.bvh().nodes.size();
        out->node_bytes = sizeof(rt::Bvh8Node);
        out->triangle_bytes = sizeof(rt::TriRecord);
        out->device_bytes = s.device_bytes();
        out->max_depth = s.bvh().depth;
        out->leaf_triangles_max = rt::kMaxLeafTris;
        out->build_seconds = s.bvh().seconds;
        s.bounds(out->bounds_min, out->bounds_max);
        out->two_level = s.two_level() ? 1u : 0u;
        out->blas_count = s.blas_count();
        out->emissive_seconds = s.emissive_seconds();
        out->bvh_device = s.bvh_on_device() ? 1u : 0u;
        out->bvh_kernel_seconds = s.bvh_kernel_seconds();
    });
}

int reina_scene_set_accel(reina_scene* scene, int mode) {
    return guard([&] {
        need(scene && scene->s, "NULL argument");
        scene->s->set_accel(mode);
    });
}

int reina_scene_set_emissive_build(reina_scene* scene, uint32_t where) {
    return guard([&] {
        need(scene && scene->s, "NULL argument");
        need(where <= REINA_EMISSIVE_DEVICE, "where must be REINA_EMISSIVE_HOST or REINA_EMISSIVE_DEVICE");
        scene->s->set_emissive_on_device(where == REINA_EMISSIVE_DEVICE);
    });
}

int reina_scene_set_bvh_build(reina_scene* scene, uint32_t where, uint32_t sah_bins, uint32_t median_depth) {
    return guard([&] {
        need(scene && scene->s, "NULL argument");
        need(where <= REINA_BVH_DEVICE, "where must be REINA_BVH_HOST or REINA_BVH_DEVICE");
        need(sah_bins == 0 || (sah_bins >= 4 && sah_bins <= 256), "sah_bins must be 0 or 4..256");
        static_assert(rt::kMaxDeviceSahBins == 64, "message below");
        need(where == REINA_BVH_HOST || sah_bins <= (uint32_t)rt::kMaxDeviceSahBins,
             "the device BVH build takes at most 64 SAH bins");
        need(median_depth <= 1024, "median_depth must be at most 1024");
        rt::BvhBuildOptions opt;
        if (sah_bins) opt.sah_bins = (int)sah_bins;
        if (median_depth) opt.median_depth = (int)median_depth;
        scene->s->set_bvh_build(where == REINA_BVH_DEVICE, opt);
    });
}

int reina_scene_export_emissive(const reina_scene* scene, EmissiveInstanceData* instances, uint32_t* n_instances,
                                float* cdf_triangles, uint64_t* n_cdf_triangles, float* cdf_instances) {
    return guard([&] {
        const rt::Scene& s = built_scene(scene);
        need(n_instances && n_cdf_triangles, "NULL count");
        const auto& d = s.emissive_data();
        const auto& ct = s.cdf_triangles();
        const auto& ci = s.cdf_instances();
        *n_instances = (uint32_t)d.size();
        *n_cdf_triangles = ct.size();
        if (instances && !d.empty()) std::memcpy(instances, d.data(), d.size() * sizeof(EmissiveInstanceData));
        if (cdf_triangles && !ct.empty()) std::memcpy(cdf_triangles, ct.data(), ct.size() * sizeof(float));
        if (cdf_instances && !ci.empty()) std::memcpy(cdf_instances, ci.data(), ci.size() * sizeof(float));
    });
}

int reina_scene_export_bvh(const reina_scene* scene, void* nodes_out, void* triangles_out) {
    return guard([&] {
        const rt::Scene& s = built_scene(scene);
        if (nodes_out) std::memcpy(nodes_out, s.bvh().nodes.data(), s.bvh().nodes.size() * sizeof(rt::Bvh8Node));
        if (triangles_out) std::memcpy(triangles_out, s.bvh().tris.data(), s.bvh().tris.size() * sizeof(rt::TriRecord));
    });
}

int reina_scene_prim_info(const reina_scene* scene, uint32_t prim, uint32_t* out_instance, uint32_t* out_primitive) {
    return guard([&] { built_scene(scene).prim_info(prim, out_instance, out_primitive); });
}

int reina_raycast_device(reina_ctx* ctx, const reina_scene* scene, const void* d_rays, uint64_t count, void* d_hits,
                         uint32_t flags, void* stream) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        need(flags <= REINA_RAY_ANY, "flags must be REINA_RAY_CLOSEST or REINA_RAY_ANY");
        need(count == 0 || (d_rays && d_hits), "NULL ray or hit buffer");
        need(((uintptr_t)d_rays % 16) == 0 && ((uintptr_t)d_hits % 16) == 0, "ray and hit buffers must be 16-byte aligned");
        need(count < (1ull << 32), "at most 2^32 - 1 rays per call");
        use_device(ctx);
        rt::launch_raycast(s.device_view(), static_cast<const rt::Ray*>(d_rays), count, static_cast<rt::Hit*>(d_hits),
                           flags == REINA_RAY_ANY, ctx->err.as<uint32_t>(), ctx->next_fetch_counter(), ctx->sm_count,
                           trace_for(ctx, flags, s.triangle_count(), count), static_cast<cudaStream_t>(stream));
        check_cuda(cudaGetLastError(), "raycast launch");
    });
}

int reina_ctx_device_error(reina_ctx* ctx, void* stream, uint32_t* out_flags) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        use_device(ctx);
        const uint32_t e = check_device_errors(ctx, static_cast<cudaStream_t>(stream));
        if (out_flags) *out_flags = e;
        if (e) fail(REINA_ERR_DEVICE, "device kernels raised error flag " + std::to_string(e) + rt::device_error_text(e));
    });
}

int reina_raycast(reina_ctx* ctx, const reina_scene* scene, const reina_ray* rays, uint64_t count, reina_hit* hits,
                  uint32_t flags) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        need(flags <= REINA_RAY_ANY, "flags must be REINA_RAY_CLOSEST or REINA_RAY_ANY");
        need(count == 0 || (rays && hits), "NULL ray or hit buffer");
        if (count == 0) return;
        use_device(ctx);
        const rt::TraceConfig cfg = trace_for(ctx, flags, s.triangle_count(), count);
        // Pinned (page-locked) host buffers: the kernel reads the rays and writes the hits in host memory
        // directly over the coherent CPU-GPU link, with no staging copies.
        const rt::Ray* zr = static_cast<const rt::Ray*>(host_device_pointer(rays, ctx->device));
        rt::Hit* zh = static_cast<rt::Hit*>(host_device_pointer(hits, ctx->device));
        if (zr && zh && count < (1ull << 32)) {
            cudaStream_t st = ctx->streams[0];
            rt::launch_raycast(s.device_view(), zr, count, zh, flags == REINA_RAY_ANY, ctx->err.as<uint32_t>(),
                               ctx->next_fetch_counter(), ctx->sm_count, cfg, st);
            check_cuda(cudaGetLastError(), "raycast launch");
            const uint32_t e = check_device_errors(ctx, st);
            if (e) fail(REINA_ERR_DEVICE, "traversal kernel raised error flag " + std::to_string(e) + rt::device_error_text(e));
            return;
        }
        ctx->rays.reserve(count * sizeof(rt::Ray));
        ctx->hits.reserve(count * sizeof(rt::Hit));
        // Pageable buffers: pipeline copies and traversal over chunks on two streams.
        const uint64_t chunk = count < (1ull << 20) ? count : std::max<uint64_t>(1ull << 19, (count + 7) / 8);
        int k = 0;
        for (uint64_t off = 0; off < count; off += chunk, ++k) {
            const uint64_t n = std::min(chunk, count - off);
            cudaStream_t st = ctx->streams[k & 1];
            rt::Ray* dr = ctx->rays.as<rt::Ray>() + off;
            rt::Hit* dh = ctx->hits.as<rt::Hit>() + off;
            check_cuda(cudaMemcpyAsync(dr, rays + off, n * sizeof(rt::Ray), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync H2D");
            rt::launch_raycast(s.device_view(), dr, n, dh, flags == REINA_RAY_ANY, ctx->err.as<uint32_t>(),
                               ctx->next_fetch_counter(), ctx->sm_count, cfg, st);
            check_cuda(cudaGetLastError(), "raycast launch");
            check_cuda(cudaMemcpyAsync(hits + off, dh, n * sizeof(rt::Hit), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync D2H");
        }
        check_cuda(cudaStreamSynchronize(ctx->streams[1]), "cudaStreamSynchronize");
        const uint32_t e = check_device_errors(ctx, ctx->streams[0]);
        if (e) fail(REINA_ERR_DEVICE, "traversal kernel raised error flag " + std::to_string(e) + rt::device_error_text(e));
    });
}

int reina_raycast_counters(reina_ctx* ctx, const reina_scene* scene, const void* d_rays, uint64_t count, uint32_t flags,
                           uint64_t* out_nodes_visited, uint64_t* out_triangles_tested, void* stream) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        need(flags <= REINA_RAY_ANY, "flags must be REINA_RAY_CLOSEST or REINA_RAY_ANY");
        need(count == 0 || d_rays, "NULL ray buffer");
        use_device(ctx);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        check_cuda(cudaMemsetAsync(ctx->counters.get(), 0, 2 * sizeof(unsigned long long), st), "cudaMemsetAsync");
        need(count < (1ull << 32), "at most 2^32 - 1 rays per call");
        rt::launch_raycast_counters(s.device_view(), static_cast<const rt::Ray*>(d_rays), count, flags == REINA_RAY_ANY,
                                    ctx->counters.as<unsigned long long>(), ctx->err.as<uint32_t>(),
                                    ctx->next_fetch_counter(), ctx->sm_count, st);
        check_cuda(cudaGetLastError(), "raycast counters launch");
        unsigned long long c[2] = {0, 0};
        check_cuda(cudaMemcpyAsync(c, ctx->counters.get(), sizeof(c), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        if (out_nodes_visited) *out_nodes_visited = c[0];
        if (out_triangles_tested) *out_triangles_tested = c[1];
    });
}

static rt::RenderOpts render_opts(const RtPushConsts* pc, const reina_render_options* o) {
    need(pc != nullptr && o != nullptr, "NULL push constants or options");
    need(o->width > 0 && o->height > 0, "image size must be positive");
    need((uint64_t)o->width * o->height <= (1ull << 28), "image too large (at most 2^28 pixels)");
    need(o->mode <= REINA_MODE_NEE_MIS, "mode must be REINA_MODE_REINA or REINA_MODE_NEE_MIS");
    need(o->env_mode <= REINA_ENV_CONSTANT, "env_mode must be REINA_ENV_SKY or REINA_ENV_CONSTANT");
    need(pc->samplesPerPixel > 0, "samplesPerPixel must be positive");
    rt::RenderOpts r;
    r.width = o->width;
    r.height = o->height;
    r.mode = o->mode;
    r.seed = o->seed;
    r.env_mode = o->env_mode;
    for (int k = 0; k < 3; ++k) r.env_color[k] = o->env_color[k];
    need((o->flags & ~(uint32_t)(REINA_RENDER_MEGAKERNEL | REINA_RENDER_PASS_BY_PASS)) == 0, "unknown render flags");
    need((o->flags & (REINA_RENDER_MEGAKERNEL | REINA_RENDER_PASS_BY_PASS)) !=
             (REINA_RENDER_MEGAKERNEL | REINA_RENDER_PASS_BY_PASS),
         "REINA_RENDER_MEGAKERNEL and REINA_RENDER_PASS_BY_PASS exclude each other");
    r.megakernel = (o->flags & REINA_RENDER_MEGAKERNEL) != 0;
    r.pass_by_pass = (o->flags & REINA_RENDER_PASS_BY_PASS) != 0;
    return r;
}

static void check_render_scene(const rt::Scene& s, const RtPushConsts* pc, const reina_render_options* o) {
    if (o->mode == REINA_MODE_NEE_MIS && s.device_view().emissive_count > 0 && !(pc->totalEmissiveWeight > 0.0f))
        fail(REINA_ERR_INVALID, "totalEmissiveWeight must be positive for NEE (use reina_scene_emissive_weight)");
}

// Validates every job, then runs waves until all are resolved.  `host`: the job buffers are host memory
// and are staged through device copies.  `force`: the traversal variant to use instead of the context's
// (or the batch autotune cache's).
static void render_batch(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, bool host, cudaStream_t st,
                         reina_render_stats* stats, const rt::TraceConfig* force = nullptr);

// One frame as the wave engine's only job (the default form of reina_render / reina_render_device).
static void render_on_engine(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* pc,
                             const reina_render_options* o, const rt::RenderOpts& r, void* accum, void* samples,
                             bool host, cudaStream_t st, reina_render_stats* stats) {
    reina_render_job job;
    std::memset(&job, 0, sizeof(job));
    job.scene = scene;
    job.push_consts = *pc;
    job.options = *o;
    job.accum_rgba32f = static_cast<float*>(accum);
    job.samples_rgb32f = static_cast<float*>(samples);
    const rt::TraceConfig trace = r.trace;
    render_batch(ctx, &job, 1, host, st, stats, &trace);
}

int reina_render_device(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* pc, const reina_render_options* o,
                        void* d_accum, void* d_samples, void* stream) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        rt::RenderOpts r = render_opts(pc, o);
        r.trace = trace_for(ctx, rt::kTuneRender, s.triangle_count(), (uint64_t)r.width * r.height);
        check_render_scene(s, pc, o);
        need(d_accum != nullptr && ((uintptr_t)d_accum % 16) == 0, "accumulation buffer must be non-NULL and 16-byte aligned");
        use_device(ctx);
        if (!r.megakernel && !r.pass_by_pass) {
            render_on_engine(ctx, scene, pc, o, r, d_accum, d_samples, false, static_cast<cudaStream_t>(stream), nullptr);
            return;
        }
        rt::render_frame(ctx->render, s.device_view(), *pc, r, static_cast<float*>(d_accum), static_cast<float*>(d_samples),
                         ctx->sm_count, static_cast<cudaStream_t>(stream), nullptr, ctx->err.as<uint32_t>());
    });
}

int reina_render_device_noalloc(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* pc,
                                const reina_render_options* o, void* d_accum, void* d_samples, void* stream) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        rt::RenderOpts r = render_opts(pc, o);
        r.trace = trace_for(ctx, rt::kTuneRender, s.triangle_count(), (uint64_t)r.width * r.height);
        check_render_scene(s, pc, o);
        need(d_accum != nullptr && ((uintptr_t)d_accum % 16) == 0, "accumulation buffer must be non-NULL and 16-byte aligned");
        use_device(ctx);
        rt::render_frame_noalloc(ctx->device, s.device_view(), *pc, r, static_cast<float*>(d_accum),
                                 static_cast<float*>(d_samples), ctx->sm_count, static_cast<cudaStream_t>(stream),
                                 ctx->err.as<uint32_t>());
    });
}

int reina_render(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* pc, const reina_render_options* o,
                 float* accum, float* samples, reina_render_stats* stats) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        rt::RenderOpts r = render_opts(pc, o);
        r.trace = trace_for(ctx, rt::kTuneRender, s.triangle_count(), (uint64_t)r.width * r.height);
        check_render_scene(s, pc, o);
        need(accum != nullptr, "accumulation buffer is NULL");
        use_device(ctx);
        if (!r.megakernel && !r.pass_by_pass) {
            render_on_engine(ctx, scene, pc, o, r, accum, samples, true, ctx->streams[0], stats);
            return;
        }
        auto t0 = std::chrono::steady_clock::now();
        const size_t P = (size_t)r.width * r.height;
        cudaStream_t st = ctx->streams[0];
        ctx->accum.reserve(P * 4 * sizeof(float));
        check_cuda(cudaMemcpyAsync(ctx->accum.get(), accum, P * 4 * sizeof(float), cudaMemcpyHostToDevice, st), "H2D accum");
        float* d_samples = nullptr;
        if (samples) {
            ctx->samples.reserve(P * pc->samplesPerPixel * 3 * sizeof(float));
            d_samples = ctx->samples.as<float>();
        }
        rt::RenderStats rs;
        rt::render_frame(ctx->render, s.device_view(), *pc, r, ctx->accum.as<float>(), d_samples, ctx->sm_count, st, &rs);
        check_cuda(cudaMemcpyAsync(accum, ctx->accum.get(), P * 4 * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H accum");
        if (samples)
            check_cuda(cudaMemcpyAsync(samples, d_samples, P * pc->samplesPerPixel * 3 * sizeof(float), cudaMemcpyDeviceToHost, st),
                       "D2H samples");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        if (rs.error) fail(REINA_ERR_DEVICE, "render kernel raised error flag " + std::to_string(rs.error) + rt::device_error_text(rs.error));
        if (stats) {
            stats->rays = rs.rays;
            stats->shadow_rays = rs.shadow_rays;
            stats->nodes_visited = rs.nodes;
            stats->triangles_tested = rs.tris;
            stats->shadow_nodes_visited = rs.shadow_nodes;
            stats->shadow_triangles_tested = rs.shadow_tris;
            stats->shaded_hits = rs.shaded;
            stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
    });
}

// Autotune key of a batch: the triangles of its distinct scenes and its total samples.
static void batch_key(const reina_render_job* jobs, uint32_t count, uint64_t* tris, uint64_t* samples) {
    std::unordered_set<const reina_scene*> seen;
    *tris = 0;
    *samples = 0;
    for (uint32_t k = 0; k < count; ++k) {
        if (seen.insert(jobs[k].scene).second) *tris += jobs[k].scene->s->triangle_count();
        *samples += (uint64_t)jobs[k].options.width * jobs[k].options.height * jobs[k].push_consts.samplesPerPixel;
    }
}

// A wave of no more slots than the batch has paths (rounded up to a power of two, at least 2^16): a
// small batch does not pay for the path state of a large wave.
static uint32_t fit_wave(uint32_t wave, uint64_t samples) {
    uint64_t fit = 1u << 16;
    while (fit < samples && fit < wave) fit <<= 1;
    return (uint32_t)std::min<uint64_t>(wave, fit);
}

// The context's batch engine, rebuilt when the wanted wave size or traversal variant changed (the
// cached autotuned ones for this batch when the context uses the cache, else the context's tuning).
static rt::BatchEngine& batch_engine(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count,
                                     const rt::TraceConfig* force) {
    uint32_t wave = ctx->wave_paths;
    rt::TraceConfig trace = ctx->wave_trace;
    rt::TuneEntry e;
    uint64_t tris = 0, samples = 0;
    batch_key(jobs, count, &tris, &samples);
    if (force) {
        trace = *force;
    } else if (ctx->autotune_mode == REINA_AUTOTUNE_CACHED &&
               ctx->tune.get(rt::kTuneBatch, rt::tune_bucket(tris), rt::tune_bucket(samples), &e)) {
        trace = e.trace;
        if (e.wave_paths) wave = e.wave_paths;
    }
    // the paths one wave can hold: every sample of a NEE+MIS job, one sample per pixel of a job in the
    // reference's mode
    uint64_t room = 0;
    for (uint32_t k = 0; k < count; ++k) {
        const uint64_t px = (uint64_t)jobs[k].options.width * jobs[k].options.height;
        room += jobs[k].options.mode == REINA_MODE_NEE_MIS ? px * jobs[k].push_consts.samplesPerPixel : px;
    }
    samples = std::min(samples, room);
    // an engine between the batch's fitted size and the wanted one is kept (a job's images do not
    // depend on how the waves are cut), so batches of changing sizes do not rebuild it each call
    const uint32_t fitted = fit_wave(wave, samples);
    if (ctx->batch && (ctx->batch->capacity() < fitted || ctx->batch->capacity() > wave ||
                       ctx->batch->lanes() != (int)ctx->wave_lanes ||
                       ctx->batch->trace().block != trace.block || ctx->batch->trace().stack != trace.stack ||
                       ctx->batch->trace().refill != trace.refill))
        ctx->batch.reset();
    if (!ctx->batch)
        ctx->batch = std::make_unique<rt::BatchEngine>(ctx->device, ctx->sm_count, fitted,
                                                       (ctx->batch_flags & REINA_BATCH_NO_GRAPHS) == 0, trace,
                                                       (int)ctx->wave_lanes);
    return *ctx->batch;
}

static void render_batch(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, bool host, cudaStream_t st,
                         reina_render_stats* stats, const rt::TraceConfig* force) {
    need(ctx != nullptr, "ctx is NULL");
    need(count == 0 || jobs != nullptr, "jobs is NULL");
    std::vector<rt::BatchJob> bj(count);
    for (uint32_t k = 0; k < count; ++k) {
        const reina_render_job& j = jobs[k];
        const rt::Scene& s = built_scene(j.scene);
        need(j.scene->ctx == ctx, "scene belongs to another context");
        const rt::RenderOpts r = render_opts(&j.push_consts, &j.options);
        need(!r.megakernel && !r.pass_by_pass, "batched jobs run the wave engine (options.flags must be 0)");
        check_render_scene(s, &j.push_consts, &j.options);
        need(j.accum_rgba32f != nullptr, "accumulation buffer is NULL");
        if (!host) need(((uintptr_t)j.accum_rgba32f % 16) == 0, "accumulation buffer must be 16-byte aligned");
        bj[k].scene = s.device_view();
        bj[k].pc = j.push_consts;
        bj[k].opt = r;
    }
    use_device(ctx);
    const auto t0 = std::chrono::steady_clock::now();
    rt::BatchEngine& eng = batch_engine(ctx, jobs, count, force);
    // host buffers are staged through device copies: the context's own staging buffers for one job,
    // buffers of the call's own for more
    std::vector<rt::DeviceBuffer> acc_own(host && count > 1 ? count : 0), smp_own(host && count > 1 ? count : 0);
    std::vector<rt::DeviceBuffer*> acc(host ? count : 0), smp(host ? count : 0);
    for (uint32_t k = 0; k < acc.size(); ++k) {
        acc[k] = count > 1 ? &acc_own[k] : &ctx->accum;
        smp[k] = count > 1 ? &smp_own[k] : &ctx->samples;
    }
    std::vector<rt::BatchJob*> ptrs(count);
    for (uint32_t k = 0; k < count; ++k) {
        const reina_render_job& j = jobs[k];
        const size_t px = (size_t)j.options.width * j.options.height;
        rt::BatchEngine::prepare(bj[k]);
        if (host) {
            acc[k]->reserve(px * 4 * sizeof(float));
            if (j.push_consts.sampleBatch > 0)
                check_cuda(cudaMemcpyAsync(acc[k]->get(), j.accum_rgba32f, px * 4 * sizeof(float), cudaMemcpyHostToDevice,
                                           st), "H2D accum");
            bj[k].d_accum = acc[k]->as<float>();
            if (j.samples_rgb32f) {
                smp[k]->reserve(px * j.push_consts.samplesPerPixel * 3 * sizeof(float));
                bj[k].d_samples = smp[k]->as<float>();
            }
        } else {
            bj[k].d_accum = static_cast<float*>(j.accum_rgba32f);
            bj[k].d_samples = static_cast<float*>(j.samples_rgb32f);
        }
        ptrs[k] = &bj[k];
    }
    const uint64_t r0 = eng.rays(), s0 = eng.shadow_rays();
    const rt::RenderStats w0 = eng.work();
    // a call that returns statistics counts the traversal work of every form
    struct Counting {
        rt::BatchEngine& e;
        Counting(rt::BatchEngine& eng, bool on) : e(eng) { e.set_counting(on); }
        ~Counting() { e.set_counting(false); }
    } counting(eng, stats != nullptr);
    eng.run_all(ptrs, st, (ctx->batch_flags & REINA_BATCH_FAIR_SHARE) == 0);
    if (host) {
        for (uint32_t k = 0; k < count; ++k) {
            const reina_render_job& j = jobs[k];
            const size_t px = (size_t)j.options.width * j.options.height;
            check_cuda(cudaMemcpyAsync(j.accum_rgba32f, acc[k]->get(), px * 4 * sizeof(float), cudaMemcpyDeviceToHost, st),
                       "D2H accum");
            if (j.samples_rgb32f)
                check_cuda(cudaMemcpyAsync(j.samples_rgb32f, smp[k]->get(), px * j.push_consts.samplesPerPixel * 3 * sizeof(float),
                                           cudaMemcpyDeviceToHost, st),
                           "D2H samples");
        }
    }
    check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (stats) {
        stats->rays = eng.rays() - r0;
        stats->shadow_rays = eng.shadow_rays() - s0;
        const rt::RenderStats& w = eng.work();
        stats->nodes_visited = w.nodes - w0.nodes;
        stats->triangles_tested = w.tris - w0.tris;
        stats->shadow_nodes_visited = w.shadow_nodes - w0.shadow_nodes;
        stats->shadow_triangles_tested = w.shadow_tris - w0.shadow_tris;
        stats->shaded_hits = w.shaded - w0.shaded;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
}

int reina_render_batch(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, reina_render_stats* stats) {
    return guard([&] { render_batch(ctx, jobs, count, true, ctx ? ctx->streams[0] : nullptr, stats); });
}

int reina_render_batch_device(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, void* stream,
                              reina_render_stats* stats) {
    return guard([&] { render_batch(ctx, jobs, count, false, static_cast<cudaStream_t>(stream), stats); });
}

int reina_postprocess_device(reina_ctx* ctx, const void* d_accum, uint32_t width, uint32_t height,
                             const BloomPushConsts* bloom, const TonemappingPushConsts* tm, void* d_rgba8, void* d_combined,
                             void* stream) {
    return guard([&] {
        need(ctx && bloom && tm, "NULL argument");
        need(d_accum && d_rgba8, "NULL image buffer");
        need(((uintptr_t)d_accum % 16) == 0 && ((uintptr_t)d_rgba8 % 4) == 0 && ((uintptr_t)d_combined % 16) == 0,
             "misaligned image buffer");
        need((uint64_t)width * height <= (1ull << 28), "image too large");
        use_device(ctx);
        rt::postprocess(ctx->post, static_cast<const float*>(d_accum), (int)width, (int)height, *bloom, *tm,
                        static_cast<uint8_t*>(d_rgba8), static_cast<float*>(d_combined), ctx->sm_count,
                        static_cast<cudaStream_t>(stream));
    });
}

int reina_postprocess(reina_ctx* ctx, const float* accum, uint32_t width, uint32_t height, const BloomPushConsts* bloom,
                      const TonemappingPushConsts* tm, uint8_t* rgba8, float* combined) {
    return guard([&] {
        need(ctx && bloom && tm && accum && rgba8, "NULL argument");
        need((uint64_t)width * height <= (1ull << 28), "image too large");
        use_device(ctx);
        const size_t n = (size_t)width * height;
        if (n == 0) return;
        cudaStream_t st = ctx->streams[0];
        ctx->accum.reserve(n * 4 * sizeof(float));
        ctx->rgba8.reserve(n * 4);
        if (combined) ctx->combined.reserve(n * 4 * sizeof(float));
        check_cuda(cudaMemcpyAsync(ctx->accum.get(), accum, n * 4 * sizeof(float), cudaMemcpyHostToDevice, st), "H2D");
        rt::postprocess(ctx->post, ctx->accum.as<float>(), (int)width, (int)height, *bloom, *tm, ctx->rgba8.as<uint8_t>(),
                        combined ? ctx->combined.as<float>() : nullptr, ctx->sm_count, st);
        check_cuda(cudaMemcpyAsync(rgba8, ctx->rgba8.get(), n * 4, cudaMemcpyDeviceToHost, st), "D2H");
        if (combined)
            check_cuda(cudaMemcpyAsync(combined, ctx->combined.get(), n * 4 * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    });
}

int reina_camera_matrices(const float pos[3], const float front[3], const float up[3], float fovy_radians, float aspect,
                          float z_near, float z_far, float inv_view[16], float inv_proj[16]) {
    return guard([&] {
        need(pos && front && up && inv_view && inv_proj, "NULL argument");
        need(aspect > 0.0f && fovy_radians > 0.0f && z_far > z_near, "bad camera parameters");
        rt::camera_matrices(pos, front, up, fovy_radians, aspect, z_near, z_far, inv_view, inv_proj);
    });
}

int reina_icosphere_counts(uint32_t level, uint64_t* out_vertices, uint64_t* out_triangles) {
    return guard([&] {
        need(level <= 12, "icosphere level must be <= 12");
        uint64_t nv, nt;
        rt::icosphere_counts(level, nv, nt);
        if (out_vertices) *out_vertices = nv;
        if (out_triangles) *out_triangles = nt;
    });
}

int reina_gen_icosphere(uint32_t level, float amplitude, uint64_t seed, float* vertices, uint32_t* indices, float* normals) {
    return guard([&] {
        need(level <= 12, "icosphere level must be <= 12");
        need(vertices && indices, "NULL output buffer");
        rt::gen_icosphere(level, amplitude, seed, vertices, indices, normals);
    });
}

int reina_geodesic_counts(uint32_t frequency, uint64_t* out_vertices, uint64_t* out_triangles) {
    return guard([&] {
        need(frequency >= 1 && frequency <= 4096, "geodesic frequency must be in 1..4096");
        uint64_t nv, nt;
        rt::geodesic_counts(frequency, nv, nt);
        if (out_vertices) *out_vertices = nv;
        if (out_triangles) *out_triangles = nt;
    });
}

int reina_gen_geodesic(uint32_t frequency, float amplitude, uint64_t seed, float* vertices, uint32_t* indices,
                       float* normals) {
    return guard([&] {
        need(frequency >= 1 && frequency <= 4096, "geodesic frequency must be in 1..4096");
        need(vertices && indices, "NULL output buffer");
        rt::gen_geodesic(frequency, amplitude, seed, vertices, indices, normals);
    });
}

int reina_gen_raycast_rays(uint32_t width, uint32_t height, const float cam_pos[3], const float cam_target[3],
                           float fovy_degrees, uint64_t n_random, const float box_min[3], const float box_max[3],
                           uint64_t seed, reina_ray* rays_out) {
    return guard([&] {
        need(cam_pos && cam_target && box_min && box_max && rays_out, "NULL argument");
        rt::gen_raycast_rays(width, height, cam_pos, cam_target, fovy_degrees, n_random, box_min, box_max, seed,
                             reinterpret_cast<rt::Ray*>(rays_out));
    });
}

// ------------------------------------------------------------------------------------------------
// Request server

int reina_server_create(reina_ctx* ctx, const reina_server_options* o, reina_server** out) {
    return guard([&] {
        need(ctx && out, "NULL argument");
        *out = nullptr;
        const uint32_t policies = REINA_SERVER_FIFO | REINA_SERVER_SHORTEST | REINA_SERVER_FAIR_SHARE;
        const uint32_t flags = o ? o->flags : 0u;
        need((flags & ~(uint32_t)(REINA_BATCH_NO_GRAPHS | policies)) == 0, "unknown server flags");
        const uint32_t policy = flags & policies;
        need((policy & (policy - 1)) == 0,
             "REINA_SERVER_SHORTEST, REINA_SERVER_FIFO and REINA_SERVER_FAIR_SHARE exclude each other");
        const float aging = o ? o->aging : 0.0f;
        need(std::isfinite(aging), "aging must be finite");
        need(!o || o->wave_lanes <= 16, "wave_lanes must be in 0..16");
        use_device(ctx);
        rt::ServerConfig cfg;
        cfg.budget = (o && o->memory_budget_bytes) ? o->memory_budget_bytes : 120000000000ull;
        cfg.max_active = (o && o->max_active_jobs) ? o->max_active_jobs : 512;
        cfg.wave_paths = o ? o->wave_paths : 0;
        cfg.lanes = o ? o->wave_lanes : 0;
        cfg.aging = aging == 0.0f ? (double)REINA_SERVER_DEFAULT_AGING : std::max(0.0, (double)aging);
        need(cfg.lanes <= 16, "wave_lanes must be in 0..16");
        cfg.graphs = !(o && (o->flags & REINA_BATCH_NO_GRAPHS));
        cfg.fifo = policy == REINA_SERVER_FIFO;
        cfg.shortest = policy == 0 || policy == REINA_SERVER_SHORTEST;
        auto s = std::make_unique<reina_server>();
        s->ctx = ctx;
        s->srv = std::make_unique<rt::Server>(ctx->device, ctx->sm_count, cfg);
        ctx->servers.insert(s.get());
        *out = s.release();
    });
}

void reina_server_destroy(reina_server* server) {
    if (!server) return;
    if (server->ctx) {
        if (server->ctx->device >= 0) cudaSetDevice(server->ctx->device);
        server->ctx->servers.erase(server);
    }
    server->srv.reset();
    for (reina_scene* sc : server->scenes) reina_scene_destroy(sc);
    delete server;
}

int reina_server_add_scene(reina_server* server, reina_scene* scene, uint32_t* out_id) {
    return guard([&] {
        need(server && scene && out_id, "NULL argument");
        need(scene->ctx == server->ctx, "scene belongs to another context");
        built_scene(scene);
        for (reina_scene* sc : server->scenes) need(sc != scene, "scene was already added");
        server->scenes.reserve(server->scenes.size() + 1);
        *out_id = server->srv->add_scene(scene->s.get());
        server->scenes.push_back(scene);
    });
}

int reina_server_submit(reina_server* server, const reina_request* req, uint64_t* out_id) {
    return guard([&] {
        need(server && req && out_id, "NULL argument");
        rt::RequestSpec spec;
        spec.scene = req->scene_id;
        spec.image_key = req->image_key;
        spec.pc = req->push_consts;
        spec.opt = render_opts(&req->push_consts, &req->options);
        spec.host_out = req->accum_rgba32f;
        *out_id = server->srv->submit(spec);
    });
}

static void to_status(const rt::RequestStatus& s, reina_request_status* out) {
    std::memset(out, 0, sizeof(*out));
    out->state = s.state;
    out->error = s.error;
    out->latency_s = s.latency_s;
    out->queue_s = s.queue_s;
    std::strncpy(out->message, s.message.c_str(), sizeof(out->message) - 1);
}

int reina_server_poll(reina_server* server, uint64_t id, reina_request_status* out) {
    return guard([&] {
        need(server && out, "NULL argument");
        to_status(server->srv->poll(id), out);
    });
}

int reina_server_wait(reina_server* server, uint64_t id, double timeout_s, reina_request_status* out) {
    return guard([&] {
        need(server && out, "NULL argument");
        to_status(server->srv->wait(id, timeout_s), out);
    });
}

int reina_server_cancel(reina_server* server, uint64_t id) {
    return guard([&] {
        need(server != nullptr, "NULL argument");
        server->srv->cancel(id);
    });
}

int reina_server_fetch_image(reina_server* server, uint64_t key, float* accum, uint32_t* w, uint32_t* h) {
    return guard([&] {
        need(server != nullptr, "NULL argument");
        server->srv->fetch_image(key, accum, w, h);
    });
}

int reina_server_get_stats(reina_server* server, reina_server_stats* out) {
    return guard([&] {
        need(server && out, "NULL argument");
        const rt::ServerStats s = server->srv->stats();
        std::memset(out, 0, sizeof(*out));
        out->submitted = s.submitted;
        out->completed = s.completed;
        out->failed = s.failed;
        out->cancelled = s.cancelled;
        out->queued = s.queued;
        out->running = s.running;
        out->latency_p50_s = s.p50;
        out->latency_p99_s = s.p99;
        out->latency_mean_s = s.mean;
        out->latency_max_s = s.max;
        out->uptime_s = s.uptime_s;
        out->busy_s = s.busy_s;
        out->first_submit_to_last_done_s = s.first_submit_to_last_done_s;
        out->rays = s.rays;
        out->shadow_rays = s.shadow_rays;
        out->waves = s.waves;
        out->scene_uploads = s.scene_uploads;
        out->scene_evictions = s.scene_evictions;
        out->image_evictions = s.image_evictions;
        out->image_restores = s.image_restores;
        out->resident_bytes = s.resident_bytes;
        out->peak_resident_bytes = s.peak_resident_bytes;
        out->budget_bytes = s.budget_bytes;
        out->reserved_bytes = s.reserved_bytes;
    });
}

// ------------------------------------------------------------------------------------------------
// Autotuner

}  // extern "C"

namespace {

// Median device time (ms) of `reps` calls of fn() on `st` after one warm-up call.
template <class F>
double time_calls(cudaStream_t st, int reps, F&& fn) {
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
    check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
    std::vector<float> ms;
    try {
        fn();
        for (int k = 0; k < reps; ++k) {
            check_cuda(cudaEventRecord(e0, st), "cudaEventRecord");
            fn();
            check_cuda(cudaEventRecord(e1, st), "cudaEventRecord");
            check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float t = 0.0f;
            check_cuda(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime");
            ms.push_back(t);
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::sort(ms.begin(), ms.end());
    return ms[ms.size() / 2];
}

// An autotuned entry as tuning fields: its launch form is the ray casts' (refill) for ray-cast kinds and
// the wavefront kernels' (wave_refill) for renders and batches; the other field is the context's.
void fill_tuning(const reina_ctx* ctx, uint32_t kind, const rt::TuneEntry& e, reina_tuning* t) {
    std::memset(t, 0, sizeof(*t));
    const bool wave = kind == rt::kTuneRender || kind == rt::kTuneBatch;
    t->refill = refill_to_abi(wave ? ctx->trace.refill : e.trace.refill);
    t->wave_refill = refill_to_abi(wave ? e.trace.refill : ctx->wave_trace.refill);
    t->trace_block = (uint32_t)e.trace.block;
    t->trace_stack = (uint32_t)e.trace.stack;
    t->trace_order = e.trace.sort ? REINA_ORDER_COHERENT : REINA_ORDER_INPUT;
    t->wave_paths = e.wave_paths ? e.wave_paths : ctx->wave_paths;
    t->batch_flags = ctx->batch_flags;
    t->wave_lanes = ctx->wave_lanes;
}

void finish_tune(reina_ctx* ctx, uint32_t kind, uint64_t tris, uint64_t size, const rt::TuneEntry& best,
                 uint32_t candidates, reina_tune_result* out) {
    const uint32_t tb = rt::tune_bucket(tris), sb = rt::tune_bucket(size);
    ctx->tune.put(kind, tb, sb, best);
    if (out) {
        std::memset(out, 0, sizeof(*out));
        fill_tuning(ctx, kind, best, &out->best);
        out->best_ms = best.best_ms;
        out->default_ms = best.default_ms;
        out->candidates = candidates;
        out->kind = kind;
        out->tri_bucket = tb;
        out->size_bucket = sb;
    }
}

// The default launch configuration of a tuning kind (ray casts: cooperative; renders and batches: grid).
bool is_default(const rt::TraceConfig& c, uint32_t kind) {
    const int refill = kind == rt::kTuneRender || kind == rt::kTuneBatch ? rt::kDefaultWaveRefill : rt::kDefaultRefill;
    return c.refill == refill && c.block == rt::kTraceBlock && c.stack == rt::kDefaultTraceStack && c.sort == 0;
}

}  // namespace

extern "C" {

int reina_autotune_raycast(reina_ctx* ctx, const reina_scene* scene, const void* d_rays, uint64_t count, void* d_hits,
                           uint32_t flags, void* stream, reina_tune_result* out) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        need(flags <= REINA_RAY_ANY, "flags must be REINA_RAY_CLOSEST or REINA_RAY_ANY");
        need(count > 0 && d_rays && d_hits, "NULL ray or hit buffer");
        need(((uintptr_t)d_rays % 16) == 0 && ((uintptr_t)d_hits % 16) == 0, "ray and hit buffers must be 16-byte aligned");
        need(count < (1ull << 32), "at most 2^32 - 1 rays per call");
        use_device(ctx);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const auto cands = rt::trace_candidates(true);
        rt::TuneEntry best;
        best.best_ms = 1e30;
        for (const rt::TraceConfig& c : cands) {
            const double ms = time_calls(st, 3, [&] {
                rt::launch_raycast(s.device_view(), static_cast<const rt::Ray*>(d_rays), count, static_cast<rt::Hit*>(d_hits),
                                   flags == REINA_RAY_ANY, ctx->err.as<uint32_t>(), ctx->next_fetch_counter(), ctx->sm_count,
                                   c, st);
                check_cuda(cudaGetLastError(), "raycast launch");
            });
            if (is_default(c, flags == REINA_RAY_ANY ? rt::kTuneRaycastAny : rt::kTuneRaycastClosest)) best.default_ms = ms;
            if (ms < best.best_ms) {
                best.best_ms = ms;
                best.trace = c;
            }
        }
        const uint32_t e = check_device_errors(ctx, st);
        if (e) fail(REINA_ERR_DEVICE, "traversal kernel raised error flag " + std::to_string(e) + rt::device_error_text(e));
        finish_tune(ctx, flags, s.triangle_count(), count, best, (uint32_t)cands.size(), out);
    });
}

int reina_autotune_render(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* pc, const reina_render_options* o,
                          reina_tune_result* out) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        const rt::Scene& s = built_scene(scene);
        rt::RenderOpts r = render_opts(pc, o);
        need(!r.megakernel, "the autotuner times the wavefront (options.flags must be 0)");
        check_render_scene(s, pc, o);
        use_device(ctx);
        RtPushConsts one = *pc;
        one.samplesPerPixel = 1;
        one.sampleBatch = 0;
        const size_t P = (size_t)r.width * r.height;
        ctx->accum.reserve(P * 4 * sizeof(float));
        cudaStream_t st = ctx->streams[0];
        const auto cands = rt::trace_candidates(false);
        rt::TuneEntry best;
        best.best_ms = 1e30;
        for (const rt::TraceConfig& c : cands) {
            r.trace = c;
            const double ms = time_calls(st, 2, [&] {
                if (r.pass_by_pass)
                    rt::render_frame(ctx->render, s.device_view(), one, r, ctx->accum.as<float>(), nullptr, ctx->sm_count,
                                     st, nullptr);
                else   // the default form: the frame as the wave engine's one job
                    render_on_engine(ctx, scene, &one, o, r, ctx->accum.get(), nullptr, false, st, nullptr);
            });
            if (is_default(c, rt::kTuneRender)) best.default_ms = ms;
            if (ms < best.best_ms) {
                best.best_ms = ms;
                best.trace = c;
            }
        }
        finish_tune(ctx, rt::kTuneRender, s.triangle_count(), P, best, (uint32_t)cands.size(), out);
    });
}

int reina_autotune_batch(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, reina_tune_result* out) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        need(count > 0 && jobs != nullptr, "no jobs");
        uint64_t tris = 0, samples = 0;
        for (uint32_t k = 0; k < count; ++k) built_scene(jobs[k].scene);
        batch_key(jobs, count, &tris, &samples);
        // up to 32 jobs (spread over the list), into scratch images, with their sample counts scaled
        // down (never below 1 per pixel) so that the subset holds about 4 of the largest candidate waves
        // or the whole batch, whichever is less: the wave size pays through the number of wave tails,
        // which a subset smaller than one wave cannot show
        const uint32_t n = std::min<uint32_t>(count, 32);
        const uint64_t kMaxWave = 1u << 23;
        std::vector<reina_render_job> sub(n);
        std::vector<rt::DeviceBuffer> scratch(n);
        uint64_t sub_samples = 0;
        for (uint32_t k = 0; k < n; ++k) {
            sub[k] = jobs[(uint64_t)k * count / n];
            sub_samples += (uint64_t)sub[k].options.width * sub[k].options.height * sub[k].push_consts.samplesPerPixel;
        }
        const double scale = std::min(1.0, (double)std::min<uint64_t>(4 * kMaxWave, samples) / (double)sub_samples);
        use_device(ctx);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t spp = sub[k].push_consts.samplesPerPixel;
            sub[k].push_consts.samplesPerPixel = std::max<uint32_t>(1, (uint32_t)std::floor(spp * scale));
            sub[k].push_consts.sampleBatch = 0;
            scratch[k].alloc((size_t)sub[k].options.width * sub[k].options.height * 4 * sizeof(float));
            sub[k].accum_rgba32f = scratch[k].get();
            sub[k].samples_rgb32f = nullptr;
        }
        const uint32_t saved_wave = ctx->wave_paths;
        const rt::TraceConfig saved_trace = ctx->wave_trace;
        const uint32_t saved_mode = ctx->autotune_mode;
        ctx->autotune_mode = REINA_AUTOTUNE_OFF;
        cudaStream_t st = ctx->streams[0];
        rt::TuneEntry best;
        best.best_ms = 1e30;
        uint32_t cands = 0;
        try {
            // candidate waves as the batch would run them (a wave beyond the batch's size shrinks to it)
            std::vector<uint32_t> waves;
            for (uint32_t w : {1u << 20, 1u << 21, 1u << 22, (uint32_t)kMaxWave})
                if (std::find(waves.begin(), waves.end(), fit_wave(w, samples)) == waves.end())
                    waves.push_back(fit_wave(w, samples));
            const uint32_t default_wave = fit_wave(REINA_DEFAULT_WAVE_PATHS, samples);
            for (uint32_t wave : waves)
                for (int refill : {rt::kDefaultWaveRefill, rt::kDefaultRefill}) {   // the grid form, the cooperative form
                    rt::TraceConfig c;
                    c.refill = refill;
                    ctx->wave_paths = wave;
                    ctx->wave_trace = c;
                    ctx->batch.reset();
                    const double ms = time_calls(st, 1, [&] { render_batch(ctx, sub.data(), n, false, st, nullptr); });
                    ++cands;
                    if (is_default(c, rt::kTuneBatch) && wave == default_wave) best.default_ms = ms;
                    if (ms < best.best_ms) {
                        best.best_ms = ms;
                        best.trace = c;
                        best.wave_paths = wave;
                    }
                }
        } catch (...) {
            ctx->wave_paths = saved_wave;
            ctx->wave_trace = saved_trace;
            ctx->autotune_mode = saved_mode;
            ctx->batch.reset();
            throw;
        }
        ctx->wave_paths = saved_wave;
        ctx->wave_trace = saved_trace;
        ctx->autotune_mode = saved_mode;
        ctx->batch.reset();
        // the subset holds only a few waves of the larger sizes, so near-ties between them are noise:
        // the default stays unless another candidate is at least 2 % faster
        if (best.default_ms > 0 && best.best_ms > 0.98 * best.default_ms) {
            best.best_ms = best.default_ms;
            best.trace = reina_ctx::wave_default();
            best.wave_paths = fit_wave(REINA_DEFAULT_WAVE_PATHS, samples);
        }
        finish_tune(ctx, rt::kTuneBatch, tris, samples, best, cands, out);
    });
}

int reina_autotune_set_mode(reina_ctx* ctx, uint32_t mode) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        need(mode <= REINA_AUTOTUNE_CACHED, "mode must be REINA_AUTOTUNE_OFF or REINA_AUTOTUNE_CACHED");
        ctx->autotune_mode = mode;
    });
}

int reina_autotune_lookup(reina_ctx* ctx, uint32_t kind, uint64_t triangles, uint64_t size, reina_tuning* out,
                          int32_t* found) {
    return guard([&] {
        need(ctx && out && found, "NULL argument");
        need(kind <= REINA_TUNE_BATCH, "unknown tune kind");
        rt::TuneEntry e;
        *found = ctx->tune.get(kind, rt::tune_bucket(triangles), rt::tune_bucket(size), &e) ? 1 : 0;
        if (*found) fill_tuning(ctx, kind, e, out);
        else std::memset(out, 0, sizeof(*out));
    });
}

int reina_autotune_save(reina_ctx* ctx, const char* path) {
    return guard([&] {
        need(ctx && path, "NULL argument");
        ctx->tune.save(path);
    });
}

int reina_autotune_load(reina_ctx* ctx, const char* path) {
    return guard([&] {
        need(ctx && path, "NULL argument");
        ctx->tune.load(path);
    });
}

// ------------------------------------------------------------------------------------------------
// Loaders, configuration, output

struct reina_save_schedule {
    rt::SaveSchedule s;
};

int reina_scene_define_object_obj(reina_scene* scene, const char* path, uint32_t* out_id) {
    return guard([&] {
        need(scene && scene->s && path && out_id, "NULL argument");
        *out_id = scene->s->define_object(rt::load_obj(path));
    });
}

int reina_scene_add_gltf(reina_scene* scene, const char* path, reina_gltf_stats* out) {
    return guard([&] {
        need(scene && scene->s && path, "NULL argument");
        if (scene->s->built()) fail(REINA_ERR_STATE, "scene is already built");
        const rt::GltfLoadStats st = rt::load_gltf(path, *scene->s);
        if (out) {
            out->meshes = st.meshes;
            out->primitives = st.primitives;
            out->instances = st.instances;
            out->skipped_primitives = st.skipped_primitives;
            out->ignored_textures = st.ignored_textures;
        }
    });
}

int reina_scene_define_texture_rgba8(reina_scene* scene, const uint8_t* rgba8, uint32_t width, uint32_t height,
                                     uint32_t* out_id) {
    return guard([&] {
        need(scene && scene->s && rgba8 && out_id, "NULL argument");
        need(width > 0 && height > 0, "texture has zero size");
        need((uint64_t)width * height <= (1ull << 28), "texture larger than 2^28 texels");
        rt::Image img;
        img.width = width;
        img.height = height;
        img.rgba.assign(rgba8, rgba8 + (size_t)width * height * 4);
        *out_id = scene->s->define_texture(std::move(img));
    });
}

int reina_scene_define_texture_file(reina_scene* scene, const char* path, uint32_t* out_id) {
    return guard([&] {
        need(scene && scene->s && path && out_id, "NULL argument");
        *out_id = scene->s->define_texture(rt::load_image(path, true));
    });
}

int reina_scene_define_texture_encoded(reina_scene* scene, const void* data, uint64_t bytes, uint32_t* out_id) {
    return guard([&] {
        need(scene && scene->s && data && out_id, "NULL argument");
        *out_id = scene->s->define_texture(rt::decode_image(static_cast<const uint8_t*>(data), (size_t)bytes));
    });
}

int reina_device_kat(reina_ctx* ctx, int kind, const float* records, uint64_t count, float* out) {
    return guard([&] {
        need(ctx != nullptr, "ctx is NULL");
        need((kind >= REINA_KAT_OFFSET && kind <= REINA_KAT_RANDOM_UNIT_VEC) || kind == REINA_KAT_SAMPLE_DISNEY_LOBE,
             "unknown kind");
        need(count == 0 || (records && out), "NULL buffer");
        need(count < (1ull << 24), "at most 2^24 cases per call");
        use_device(ctx);
        if (count == 0) return;
        rt::DeviceBuffer d_rec(count * rt::kKatRecordFloats * sizeof(float)), d_out(count * 4 * sizeof(float));
        check_cuda(cudaMemcpy(d_rec.get(), records, d_rec.bytes(), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        rt::launch_kat(kind, d_rec.as<float>(), (uint32_t)count, d_out.as<float>(), nullptr);
        check_cuda(cudaGetLastError(), "kat launch");
        check_cuda(cudaMemcpy(out, d_out.get(), d_out.bytes(), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    });
}

int reina_scene_export_two_level(const reina_scene* scene, void* records, uint32_t* refs, uint32_t* ninst,
                                 uint32_t* nrefs) {
    return guard([&] {
        const rt::Scene& s = built_scene(scene);
        const auto& it = s.instance_records();
        const auto& r = s.tlas_refs();
        if (ninst) *ninst = (uint32_t)it.size();
        if (nrefs) *nrefs = (uint32_t)r.size();
        if (records) std::memcpy(records, it.data(), it.size() * sizeof(rt::InstanceTrav));
        if (refs) std::memcpy(refs, r.data(), r.size() * sizeof(uint32_t));
    });
}

int reina_scene_export_properties(const reina_scene* scene, InstanceProperties* out, uint32_t capacity,
                                  uint32_t* out_count) {
    return guard([&] {
        need(scene && scene->s && out_count, "NULL argument");
        const std::vector<InstanceProperties>& p = scene->s->instance_properties();
        *out_count = (uint32_t)p.size();
        if (out) {
            need(capacity >= p.size(), "capacity smaller than the number of records");
            std::memcpy(out, p.data(), p.size() * sizeof(InstanceProperties));
        }
    });
}

int reina_scene_texture_count(const reina_scene* scene, uint32_t* out) {
    return guard([&] {
        need(scene && scene->s && out, "NULL argument");
        *out = (uint32_t)scene->s->texture_count();
    });
}

int reina_scene_export_texture(const reina_scene* scene, uint32_t id, uint32_t* w, uint32_t* h, uint8_t* rgba8,
                               uint64_t cap) {
    return guard([&] {
        need(scene && scene->s && w && h, "NULL argument");
        const rt::Image& img = scene->s->texture(id);
        *w = img.width;
        *h = img.height;
        if (rgba8) {
            need(cap >= img.rgba.size(), "rgba8_capacity smaller than width*height*4");
            std::memcpy(rgba8, img.rgba.data(), img.rgba.size());
        }
    });
}

int reina_decode_image(const void* data, uint64_t bytes, uint32_t* w, uint32_t* h, uint8_t* rgba8, uint64_t cap) {
    return guard([&] {
        need(data && w && h, "NULL argument");
        const rt::Image img = rt::decode_image(static_cast<const uint8_t*>(data), (size_t)bytes);
        *w = img.width;
        *h = img.height;
        if (rgba8) {
            need(cap >= img.rgba.size(), "rgba8_capacity smaller than width*height*4");
            std::memcpy(rgba8, img.rgba.data(), img.rgba.size());
        }
    });
}

int reina_scene_object_count(const reina_scene* scene, uint32_t* out) {
    return guard([&] {
        need(scene && scene->s && out, "NULL argument");
        *out = (uint32_t)scene->s->object_count();
    });
}

int reina_scene_export_object(const reina_scene* scene, uint32_t id, float* v, uint64_t* nv, uint32_t* idx, uint64_t* ni,
                              float* tbn, uint64_t* nt, float* uv, uint64_t* nuv) {
    return guard([&] {
        need(scene && scene->s, "NULL argument");
        const rt::ModelData& m = scene->s->model(id);
        if (nv) *nv = m.vertices.size() / 4;
        if (ni) *ni = m.indices.size();
        if (nt) *nt = m.tbns.size() / 9;
        if (nuv) *nuv = m.tex_coords.size() / 2;
        if (v) std::memcpy(v, m.vertices.data(), m.vertices.size() * sizeof(float));
        if (idx) std::memcpy(idx, m.indices.data(), m.indices.size() * sizeof(uint32_t));
        if (tbn) std::memcpy(tbn, m.tbns.data(), m.tbns.size() * sizeof(float));
        if (uv) std::memcpy(uv, m.tex_coords.data(), m.tex_coords.size() * sizeof(float));
    });
}

int reina_config_load(const char* path, reina_config* out) {
    return guard([&] {
        need(path && out, "NULL argument");
        const rt::RunConfig c = rt::load_config(path);
        if (c.save_on_samples.size() > REINA_CONFIG_MAX_SAVES || c.save_on_times.size() > REINA_CONFIG_MAX_SAVES)
            fail(REINA_ERR_IO, std::string(path) + ": more than " + std::to_string(REINA_CONFIG_MAX_SAVES) + " save points");
        std::memset(out, 0, sizeof(*out));
        out->focus_dist = c.focus_dist;
        out->defocus_multiplier = c.defocus_multiplier;
        out->samples_per_pixel = c.samples_per_pixel;
        out->max_bounces = c.max_bounces;
        out->direct_clamp = c.direct_clamp;
        out->indirect_clamp = c.indirect_clamp;
        out->bloom.radius = c.bloom_radius;
        out->bloom.threshold = c.bloom_threshold;
        out->bloom.intensity = c.bloom_intensity;
        out->tonemap.exposure = c.exposure;
        out->save_on_samples_count = (uint32_t)c.save_on_samples.size();
        out->save_on_times_count = (uint32_t)c.save_on_times.size();
        for (size_t k = 0; k < c.save_on_samples.size(); ++k) out->save_on_samples[k] = c.save_on_samples[k];
        for (size_t k = 0; k < c.save_on_times.size(); ++k) out->save_on_times[k] = c.save_on_times[k];
        out->width = c.width;
        out->height = c.height;
        out->seed = c.seed;
        out->mode = c.mode;
        need(c.scene_path.size() < sizeof(out->scene_path), "scene.path longer than 511 bytes");
        std::memcpy(out->scene_path, c.scene_path.c_str(), c.scene_path.size() + 1);
        for (int k = 0; k < 3; ++k) {
            out->camera_pos[k] = c.camera_pos[k];
            out->look_at[k] = c.look_at[k];
        }
        out->fov_degrees = c.fov_degrees;
    });
}

int reina_save_schedule_create(const reina_config* c, reina_save_schedule** out) {
    return guard([&] {
        need(c && out, "NULL argument");
        need(c->save_on_samples_count <= REINA_CONFIG_MAX_SAVES && c->save_on_times_count <= REINA_CONFIG_MAX_SAVES,
             "too many save points");
        std::vector<int64_t> smp(c->save_on_samples, c->save_on_samples + c->save_on_samples_count);
        std::vector<double> tm(c->save_on_times, c->save_on_times + c->save_on_times_count);
        *out = new reina_save_schedule{rt::SaveSchedule(std::move(smp), std::move(tm))};
    });
}

void reina_save_schedule_destroy(reina_save_schedule* s) { delete s; }

int reina_save_schedule_next(reina_save_schedule* s, uint64_t samples, double seconds, char* name, size_t cap) {
    return guard([&] {
        need(s && name, "NULL argument");
        need(cap >= 64, "name buffer must hold at least 64 bytes");
        const std::string n = s->s.next(samples, seconds);
        need(n.size() < cap, "name buffer too small");
        std::memcpy(name, n.c_str(), n.size() + 1);
    });
}

int reina_write_png(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h) {
    return guard([&] {
        need(path && rgba8, "NULL argument");
        rt::write_png(path, rgba8, w, h);
    });
}

}  // extern "C"
