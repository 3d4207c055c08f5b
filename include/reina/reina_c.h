/*
 * reina_c.h — C ABI of the GB300 trace path (BVH build -> traversal -> wavefront integrator ->
 * accumulation -> post-process) that stands in for Reina's Vulkan ray-tracing pipeline.
 *
 * The entry points mirror the reference's scene API and per-frame calls one for one; each declaration
 * names the reference interface (file:line, relative to the reina-vk project root) that it replaces.
 * Conventions:
 *   - every function returns an int status: REINA_OK (0) or a negative REINA_ERR_* code; the message of
 *     the last failure on the calling thread is returned by reina_last_error().  No C++ exception
 *     crosses this boundary (the reference throws std::runtime_error, caught in src/main.cpp:11-14).
 *   - handles are opaque and owned by the library; release them with the matching *_destroy call.
 *   - "host" buffers are plain CPU pointers; "device" buffers are CUDA device pointers on the context's
 *     GPU; `stream` arguments are cudaStream_t values passed as void* (NULL = the legacy default stream).
 */
#ifndef REINA_C_H
#define REINA_C_H

#include <stddef.h>
#include <stdint.h>

#include "polyglot.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------------------ */
/* Status codes                                                                                      */
/* ------------------------------------------------------------------------------------------------ */
enum {
    REINA_OK = 0,
    REINA_ERR_INVALID = -1,      /* bad argument (null pointer, out-of-range id, size mismatch) */
    REINA_ERR_CUDA = -2,         /* a CUDA runtime call failed */
    REINA_ERR_OOM = -3,          /* device or host allocation failed */
    REINA_ERR_STATE = -4,        /* call made in the wrong state (e.g. add to a built scene) */
    REINA_ERR_IO = -5,           /* file could not be read or parsed */
    REINA_ERR_NO_EMISSIVE = -6,  /* scene has no emissive geometry (src/scene/Instances.cpp:125-127) */
    REINA_ERR_DEVICE = -7,       /* a kernel raised its error flag (e.g. traversal stack overflow) */
    REINA_ERR_BUDGET = -8        /* request does not fit the device-memory admission budget */
};

/* Message of the last failed call on this thread ("" if none).  The pointer stays valid until the
 * next failing call on the same thread. */
const char* reina_last_error(void);

/* Library version string, e.g. "reina-gb300 0.1 sm_103a". */
const char* reina_version(void);

/* ------------------------------------------------------------------------------------------------ */
/* Context                                                                                           */
/* ------------------------------------------------------------------------------------------------ */
typedef struct reina_ctx reina_ctx;

typedef struct reina_ctx_options {
    int32_t device;              /* CUDA device ordinal; the context makes it current on each call.
                                  * -1 = host-only context: scenes are assembled and their BVH built
                                  * on the CPU, nothing is uploaded and GPU calls fail. */
    uint32_t flags;              /* reserved, 0 */
} reina_ctx_options;

/* Creates the per-GPU context (replaces the Vulkan instance/device set-up of src/Reina.cpp:61-74). */
int reina_ctx_create(const reina_ctx_options* options, reina_ctx** out_ctx);
void reina_ctx_destroy(reina_ctx* ctx);
/* Number of streaming multiprocessors of the context's GPU (0 if unknown). */
int reina_ctx_sm_count(const reina_ctx* ctx);

/* Launch parameters of the traversal kernels and of batched renders (no counterpart in the reference,
 * whose traversal and scheduling belong to the Vulkan implementation).  Every setting gives the same results; only speed
 * differs.  0 selects the default of a field.
 *   refill: the traversal launch form.  1..32 (0 = the default, 8): the warp-cooperative persistent form
 *            (flat scenes; block 128, stack 12): warps keep 32 rays in flight, take new rays once `refill`
 *            of their lanes are idle, and share each step's triangle tests and the finished rays' hit
 *            refinement over all 32 lanes; REINA_REFILL_GRID: one thread per ray (the grid form, the
 *            only form of two-level scenes, which use it whatever this field says).  On the
 *            1.3M-triangle ray cast (2,097,152 rays) closest hit 0.58 ms cooperative against 0.82 ms
 *            grid, any hit 0.36 against 0.51 ms.  Ray casts only: the wavefront kernels of frames and
 *            batches take wave_refill, whose default is the grid form (a 1920x1080 64-spp frame of that
 *            scene 318 ms grid against 352 ms cooperative, a 256x256 Cornell room 2.48 against 3.79 ms).
 *   trace_block: threads per block of the grid-form traversal kernels (ray cast, wavefront extend and
 *            shadow): 64, 128 or 256 (default 128).  Grid form only.
 *   trace_stack: shared-memory traversal stack entries per thread, 8, 12 or 16 (default 12); deeper
 *            levels spill to local memory.
 *   trace_order: the order a grid-form ray cast traces its rays in (below).
 *   wave_paths: path slots of one wave of a batched render or frame (0 = REINA_DEFAULT_WAVE_PATHS);
 *            the path state costs 164 bytes per slot and wave in flight (wave_lanes): the waves run on
 *            streams of their own, so that one wave's last bounces (few long paths) overlap the next
 *            waves' first ones.  A wave holds any number of samples of a pixel of a NEE+MIS job and at
 *            most one of a job in the reference's mode; a batch gets no more slots than one wave can
 *            hold of it, rounded up to a power of two (at least 2^16); an engine already built with
 *            more slots than that (up to wave_paths) is reused.
 *   batch_flags: REINA_BATCH_NO_GRAPHS launches each wave's kernels one by one instead of replaying a
 *            captured CUDA graph.  Waves are packed with the jobs in list order, each taking all it can
 *            use (one sample of each of its pixels), so that a wave holds few scenes and their data
 *            stays in L2 (on a 256-scene batch 9.06 s against 9.40 s for an equal share per job);
 *            REINA_BATCH_FAIR_SHARE gives every unfinished job an equal share of each wave instead.
 *            Neither changes an image.
 * Changing wave_paths, batch_flags, wave_refill, trace_block or trace_stack releases the batch engine; the
 * next batched call rebuilds it.  The request server's engine uses the defaults. */
typedef struct reina_tuning {
    uint32_t refill;
    uint32_t wave_paths;
    uint32_t batch_flags;
    uint32_t trace_block;
    uint32_t trace_stack;
    uint32_t trace_order;        /* ray casts, grid form: REINA_ORDER_INPUT (default) or REINA_ORDER_COHERENT */
    uint32_t wave_lanes;         /* waves in flight in batched renders and frames, 1..16
                                  * (0 = REINA_DEFAULT_WAVE_LANES) */
    uint32_t wave_refill;        /* launch form of the wavefront extension and shadow kernels (frames,
                                  * batches): like `refill`, but 0 = the default REINA_REFILL_GRID */
} reina_tuning;
/* REINA_ORDER_INPUT traces ray i on thread i.  REINA_ORDER_COHERENT first bins the rays by direction
 * octant and origin cell (Morton order on an 8^3 grid over the origins' bounds) and traces them in that
 * order, so that neighbouring threads follow similar paths; hits still go to each ray's own slot.  It
 * costs four small kernels and 8 bytes of stream-ordered scratch per ray, and pays only for incoherent
 * ray sets (on the 1.3M-triangle workload: random half 0.513 vs 0.525 ms, camera half 0.49 vs 0.46 ms);
 * the autotuner tries both. */
enum { REINA_ORDER_INPUT = 0, REINA_ORDER_COHERENT = 1 };
enum { REINA_REFILL_GRID = 255 };
/* Waves of 2^21 slots, 8 in flight (2.75 GB of path state).  Every wave ends in a tail of a few long
 * paths at low occupancy (late bounces are latency-bound chains of node fetches), which the other waves
 * in flight fill.  On a 256-scene batch (3.1 G paths): one wave in flight 12.94 s at 2^21 slots and
 * 9.05 s at 2^24; two 7.75 s (2^23); four 7.27 s (2^22); eight 7.07 s (2^21); sixteen 7.02 s (2^20).
 * On a 1920x1080, 64 spp, 12-bounce frame (waves of one sample per pixel): one 0.599 s, two 0.400 s,
 * four 0.331 s, eight 0.324 s.  The server's waves are as large, with fewer in flight
 * (REINA_SERVER_WAVE_LANES) so that new requests join sooner. */
enum {
    REINA_DEFAULT_WAVE_PATHS = 2097152,
    REINA_DEFAULT_WAVE_LANES = 8,
    REINA_SERVER_WAVE_PATHS = 2097152,
    REINA_SERVER_WAVE_LANES = 4
};
enum { REINA_BATCH_NO_GRAPHS = 1, REINA_BATCH_FAIR_SHARE = 2 };
int reina_ctx_set_tuning(reina_ctx* ctx, const reina_tuning* tuning);
int reina_ctx_get_tuning(const reina_ctx* ctx, reina_tuning* out_tuning);

/* ------------------------------------------------------------------------------------------------ */
/* Scene API  (src/scene/Scene.h:62-138)                                                             */
/* ------------------------------------------------------------------------------------------------ */
typedef struct reina_scene reina_scene;

/* ModelData (src/scene/Models.h:23-30), passed as borrowed arrays; the scene copies them. */
typedef struct reina_model_data {
    const float* vertices;       /* 4 floats per vertex (x, y, z, w = 1) */
    uint64_t vertex_count;
    const uint32_t* indices;     /* 3 per triangle, relative to this model */
    uint64_t index_count;
    const float* tbns;           /* 9 floats per entry: mat3 column-major, columns T, B, N */
    uint64_t tbn_count;
    const uint32_t* tbn_indices; /* 3 per triangle */
    uint64_t tbn_index_count;
    const float* tex_coords;     /* 2 floats per entry; may be NULL */
    uint64_t tex_coord_count;
    const uint32_t* tex_indices; /* 3 per triangle; may be NULL */
    uint64_t tex_index_count;
} reina_model_data;

/* Material (src/scene/Scene.h:21-46).  material_idx: 0 Lambertian, 1 metal, 2 dielectric, 3 Disney
 * (the shader-binding-table offset of src/tools/vktools.cpp:483). */
typedef struct reina_material {
    uint32_t material_idx;
    int32_t texture_id;
    int32_t normal_map_id;
    int32_t bump_map_id;
    float albedo[3];
    float emission[3];
    float roughness;
    float ior;
    uint32_t interp_normals;
    float absorption;
    uint32_t cull_backface;
    float anisotropic;
    float subsurface;
    float clearcoat_gloss;
    float sheen_tint[3];
    float specular_tint[3];
    float metallic;
    float clearcoat;
    float specular_transmission;
    float sheen;
} reina_material;

/* Scene::Scene() */
int reina_scene_create(reina_ctx* ctx, reina_scene** out_scene);
void reina_scene_destroy(reina_scene* scene);

/* Scene::defineObject(const ModelData&)  (src/scene/Scene.h:78, src/scene/Models.cpp:24-92) */
int reina_scene_define_object(reina_scene* scene, const reina_model_data* model, uint32_t* out_object_id);

/* Scene::addInstance(objectID, transform, material)  (src/scene/Scene.h:114, Scene.cpp:27-54).
 * transform: 16 floats, column-major object-to-world matrix (glm::mat4). */
int reina_scene_add_instance(reina_scene* scene, uint32_t object_id, const float transform[16],
                             const reina_material* material);

/* Extension for per-face materials: face f of the object uses materials[face_material[f]].  Each
 * distinct material becomes one InstanceProperties record; emission of per-face materials must be 0. */
int reina_scene_add_instance_per_face(reina_scene* scene, uint32_t object_id, const float transform[16],
                                      const reina_material* materials, uint32_t material_count,
                                      const uint32_t* face_material);

/* Scene::build(...)  (src/scene/Scene.cpp:56-125): assembles the global vertex/index/TBN/UV buffers,
 * InstanceProperties and the emissive CDFs, builds the binned-SAH BVH collapsed to quantized BVH8
 * nodes (replacing the BLAS/TLAS builds of src/graphics/Blas.cpp:8-124, src/tools/vktools.cpp:460-596)
 * and uploads everything to the GPU.  Returns REINA_ERR_NO_EMISSIVE when `require_emissive` is set
 * and the scene has no emissive instance (src/scene/Instances.cpp:125-127). */
int reina_scene_build(reina_scene* scene, uint32_t require_emissive);

/* Scene::getEmissiveWeight()  (src/scene/Scene.h:118): total emissive weight Σ area·luminance. */
float reina_scene_emissive_weight(const reina_scene* scene);

/* Acceleration structure of a scene, chosen before reina_scene_build:
 *   REINA_ACCEL_AUTO       two levels when instancing repeats models (the flattened triangle count is at
 *                          least twice the count of one copy per model) and every transform is invertible
 *   REINA_ACCEL_FLAT       one BVH8 over all instances' world-space triangles
 *   REINA_ACCEL_TWO_LEVEL  the reference's structure (src/scene/Scene.cpp:93-116): a top-level BVH8 over
 *                          instances and one bottom-level BVH8 per model in object space; rays enter an
 *                          instance through its inverse transform (REINA_ERR_INVALID at the build if a
 *                          transform is singular).
 * Hit ids are global triangle ids either way (instance's first triangle + triangle within the model). */
enum { REINA_ACCEL_AUTO = 0, REINA_ACCEL_FLAT = 1, REINA_ACCEL_TWO_LEVEL = 2 };
int reina_scene_set_accel(reina_scene* scene, int mode);

/* Where reina_scene_build computes the emissive CDFs (Instance::computeCDF, src/scene/Instance.cpp:15-53)
 * and their duplicate search (Instances.cpp:52-90): REINA_EMISSIVE_HOST (default) or REINA_EMISSIVE_DEVICE,
 * the scene's GPU (REINA_ERR_STATE at the build on a host-only context).  The device build evaluates the
 * same expressions in the same order with explicit rounding — vertex transform, triangle areas and
 * normalization in parallel, each instance's running sum in one thread, pairwise comparison in parallel
 * — so both give the same bits. */
enum { REINA_EMISSIVE_HOST = 0, REINA_EMISSIVE_DEVICE = 1 };
int reina_scene_set_emissive_build(reina_scene* scene, uint32_t where);

/* Where reina_scene_build builds the triangle BVHs (the BLAS builds of src/graphics/Blas.cpp:41-113 and,
 * for flat scenes, the whole-scene structure): REINA_BVH_HOST (default, multithreaded C++) or
 * REINA_BVH_DEVICE, the scene's GPU (REINA_ERR_STATE at the build on a host-only context).  The top level
 * of a two-level scene (instance boxes) is always built on the host.  Both builders run the same binned
 * SAH, collapse and quantization with the same explicitly rounded arithmetic and write byte-identical
 * nodes and triangle records.  `sah_bins`: bins per axis (0: 32; the device build takes 4..64);
 * `median_depth`: binary depth from which every split is an object median (0: 48). */
enum { REINA_BVH_HOST = 0, REINA_BVH_DEVICE = 1 };
int reina_scene_set_bvh_build(reina_scene* scene, uint32_t where, uint32_t sah_bins, uint32_t median_depth);

/* The packed emissive sampling data of a built scene (the buffers NEE reads, Instances.cpp:92-114): one
 * EmissiveInstanceData per emissive instance, the concatenated per-instance triangle CDFs and the
 * instance CDF.  Pass NULL arrays to get the counts first; a non-NULL array must hold its count. */
int reina_scene_export_emissive(const reina_scene* scene, EmissiveInstanceData* instances, uint32_t* n_instances,
                                float* cdf_triangles, uint64_t* n_cdf_triangles, float* cdf_instances);

typedef struct reina_scene_stats {
    uint64_t triangle_count;
    uint64_t instance_count;
    uint64_t node_count;         /* BVH8 nodes */
    uint64_t node_bytes;         /* bytes of one BVH8 node (80) */
    uint64_t triangle_bytes;     /* bytes of one traversal triangle record (48) */
    uint64_t device_bytes;       /* device memory held by the scene */
    uint32_t max_depth;          /* depth of the BVH8 tree (root = 1) */
    uint32_t leaf_triangles_max; /* largest triangle count of one leaf child (<= 3) */
    double build_seconds;        /* wall time of the BVH build (host or device builder) */
    float bounds_min[3];
    float bounds_max[3];
    uint32_t two_level;          /* 1: top level over instances + bottom levels per model */
    uint32_t blas_count;         /* bottom-level BVHs (two-level scenes) */
    double emissive_seconds;     /* wall time of the emissive CDF build and its duplicate search */
    uint32_t bvh_device;         /* 1: triangle BVHs built on the GPU (REINA_BVH_DEVICE) */
    uint32_t pad0;
    double bvh_kernel_seconds;   /* device builds: GPU time of their kernels (CUDA events) */
} reina_scene_stats;
int reina_scene_get_stats(const reina_scene* scene, reina_scene_stats* out_stats);

/* Copies the scene's BVH8 nodes (node_count * 80 bytes) and traversal triangles (triangle_count * 48
 * bytes) to host buffers, for inspection and structural checks.  Either pointer may be NULL. */
int reina_scene_export_bvh(const reina_scene* scene, void* nodes_out, void* triangles_out);

/* Two-level scenes: copies the per-instance traversal records (64 bytes each: world-to-object matrix as
 * 12 floats row-major 3x4, bottom-level root node index, first global triangle id, 2 words of padding)
 * and the top-level leaf entries (instance ids; a top-level leaf child's offset indexes them from the
 * node's tri_base).  Either pointer may be NULL; the counts are written (0 for a flat scene). */
int reina_scene_export_two_level(const reina_scene* scene, void* instance_records, uint32_t* tlas_refs,
                                 uint32_t* out_instance_count, uint32_t* out_ref_count);

/* Copies the scene's InstanceProperties records (polyglot.h; the records the closest-hit shaders read,
 * built as src/scene/Scene.cpp:27-54 builds them) to `out` (capacity records; NULL to query the count
 * only).  *out_count receives the number of records.  Available before and after the build. */
int reina_scene_export_properties(const reina_scene* scene, InstanceProperties* out, uint32_t capacity,
                                  uint32_t* out_count);

/* Maps a global triangle id (as returned in reina_hit.prim) to (instance index, primitive index
 * within the instance's object) — the pair (gl_InstanceID, gl_PrimitiveID) of the reference. */
int reina_scene_prim_info(const reina_scene* scene, uint32_t prim, uint32_t* out_instance,
                          uint32_t* out_primitive);

/* ------------------------------------------------------------------------------------------------ */
/* Ray casting (closest hit / any hit) — replaces traceRayEXT (shaders/raytrace/raytrace.rgen.glsl:  */
/* 159-171, closest hit, opaque) and the shadow query of shaders/raytrace/nee.h.glsl:126-144          */
/* (gl_RayFlagsTerminateOnFirstHitEXT).                                                              */
/* ------------------------------------------------------------------------------------------------ */
typedef struct reina_ray {       /* 32 bytes */
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} reina_ray;

typedef struct reina_hit {       /* 16 bytes */
    uint32_t prim;               /* global triangle id, 0xFFFFFFFF = miss */
    float t;
    float u;                     /* barycentric weight of vertex 1 (gl hit attribute .x) */
    float v;                     /* barycentric weight of vertex 2 (gl hit attribute .y) */
} reina_hit;

enum {
    REINA_RAY_CLOSEST = 0,       /* closest hit; ties in t go to the lower triangle id */
    REINA_RAY_ANY = 1            /* first hit found in [tmin, tmax]; terminate traversal */
};

/* Host buffers (blocking).  Page-locked buffers of the context's device (cudaHostAlloc /
 * cudaHostRegister) are read and written in place by the kernel over the coherent CPU-GPU link; other
 * buffers are copied to the GPU and back in chunks overlapped with the traversal. */
int reina_raycast(reina_ctx* ctx, const reina_scene* scene, const reina_ray* rays, uint64_t count,
                  reina_hit* hits, uint32_t flags);

/* Device buffers: enqueues the trace on `stream` and returns without synchronizing. */
int reina_raycast_device(reina_ctx* ctx, const reina_scene* scene, const void* d_rays, uint64_t count,
                         void* d_hits, uint32_t flags, void* stream);

/* Traversal statistics for the same rays (a separate counting build of the traversal kernel, never
 * used for timing): per-ray BVH8 nodes visited and triangles tested, summed into the two outputs. */
int reina_raycast_counters(reina_ctx* ctx, const reina_scene* scene, const void* d_rays, uint64_t count,
                           uint32_t flags, uint64_t* out_nodes_visited, uint64_t* out_triangles_tested,
                           void* stream);

/* ------------------------------------------------------------------------------------------------ */
/* Rendering — replaces Reina::traceRays (src/Reina.cpp:425-470), i.e. vkCmdTraceRaysKHR over the     */
/* image with the raygen shader of shaders/raytrace/raytrace.rgen.glsl:250-285.                       */
/* ------------------------------------------------------------------------------------------------ */
enum {
    REINA_MODE_REINA = 0,        /* the reference's integrator as shipped: NEE off (raytrace.rgen.glsl:146),
                                  * per-pixel seed (sampleBatch*H + y)*W + x carried across samples */
    REINA_MODE_NEE_MIS = 1       /* NEE on Lambertian and Disney hits with power-heuristic MIS; per-path
                                  * seed hash(pixel, sampleBatch*spp + sample, seed) */
};
enum {
    REINA_ENV_SKY = 0,           /* sky gradient of shaders/raytrace/raytrace.rmiss.glsl:10-19 */
    REINA_ENV_CONSTANT = 1       /* constant environment radiance env_color */
};

typedef struct reina_render_options {
    uint32_t width;
    uint32_t height;
    uint32_t mode;               /* REINA_MODE_* */
    uint32_t seed;               /* key of the per-path seeds in REINA_MODE_NEE_MIS */
    uint32_t env_mode;           /* REINA_ENV_* */
    float env_color[3];
    uint32_t flags;              /* REINA_RENDER_* */
} reina_render_options;

enum {
    REINA_RENDER_MEGAKERNEL = 1,   /* plain form: one kernel with one thread per pixel running all of its
                                    * samples and segments (the reference's raygen structure), instead of
                                    * the wavefront of queue-driven kernels */
    REINA_RENDER_PASS_BY_PASS = 2  /* the wavefront one sample pass at a time with direct kernel launches
                                    * (no CUDA graphs, no overlap between passes), instead of the wave
                                    * engine of the batched renders with the frame as its one job */
};
/* Without a flag a frame runs on the context's wave engine (reina_render_batch with one job): waves
 * of its samples (several per pixel in REINA_MODE_NEE_MIS, one per pixel in REINA_MODE_REINA), eight in
 * flight on their own streams (tuning.wave_lanes), each replayed from a CUDA graph — on the 1920x1080,
 * 64 spp, 12-bounce frame 0.32 s against 0.59 s pass by pass.  The three forms give the same images. */
/* The grid-form traversal variant of a frame comes from the render autotune cache (REINA_AUTOTUNE_CACHED)
 * or the context's tuning; the cooperative form (the default) runs the extension and shadow kernels of
 * both the wave engine and the pass-by-pass form for flat scenes. */

typedef struct reina_render_stats {
    uint64_t rays;               /* closest-hit rays traced (path segments) */
    uint64_t shadow_rays;        /* any-hit shadow rays traced */
    double seconds;              /* wall time of the call */
    /* traversal work of the wave engine's extension and shadow kernels (0 where a frame ran pass by pass or
     * as the megakernel): BVH8 nodes visited and triangles tested by the path segments and by the shadow
     * rays, and the hits shaded by a material kernel.  A call that fills these runs the counting kernels
     * of its traversal form (the same traversal, so the same image). */
    uint64_t nodes_visited;
    uint64_t triangles_tested;
    uint64_t shadow_nodes_visited;
    uint64_t shadow_triangles_tested;
    uint64_t shaded_hits;
} reina_render_stats;

/* One frame of the wavefront path tracer: push_consts->samplesPerPixel samples per pixel, at most
 * push_consts->maxBounces segments per sample, samples clamped to [0, directClamp] with NaN samples
 * dropped, and the frame's mean blended into `accum_rgba32f` (width*height RGBA32F, host memory) as
 * (prev*sampleBatch + mean)/(sampleBatch + 1) when sampleBatch > 0 (raytrace.rgen.glsl:264-284).
 * `samples_rgb32f` (optional, width*height*spp*3 floats) receives every sample's clamped colour. */
int reina_render(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* push_consts,
                 const reina_render_options* options, float* accum_rgba32f, float* samples_rgb32f,
                 reina_render_stats* stats);

/* Same on device buffers, enqueued on `stream` without synchronizing.  d_samples may be NULL. */
int reina_render_device(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* push_consts,
                        const reina_render_options* options, void* d_accum_rgba32f, void* d_samples_rgb32f,
                        void* stream);

/* Device error flags of the asynchronous entry points (reina_raycast_device, reina_render_device,
 * reina_render_device_noalloc).  Their kernels never trap: a traversal that overflows its stack (bit 1)
 * or runs past the traversal step limit (bit 2), or — in the checked build — an out-of-range queue index
 * (bit 4), sets a bit in the context's device error word and the ray or path ends.  This call orders a
 * read of that word after the work queued on `stream`, waits for it, writes the bits to *out_flags
 * (optional), clears the word and returns REINA_ERR_DEVICE if any bit was set.  The synchronous entry
 * points check the word themselves and fail with REINA_ERR_DEVICE.  Reference: the run loop's errors
 * surface as exceptions caught in main (src/main.cpp:11-14). */
int reina_ctx_device_error(reina_ctx* ctx, void* stream, uint32_t* out_flags);

/* Allocation-free render.  No counterpart in the reference: this entry point exists for callers that
 * cannot call cudaMalloc while they run — a host whose allocator owns all device memory and gives none
 * to plug-ins, a process whose device-memory budget is already handed out, or a frame loop that cannot
 * afford the device-wide synchronization a cudaMalloc may cause.  It renders exactly like
 * reina_render_device, but keeps the wavefront's path state and queues in a fixed array inside the
 * library (REINA_NOALLOC_MAX_PIXELS pixels, 11.3 MB, held by every GPU that loads the library until
 * the process exits) and calls no cudaMalloc, cudaFree or other allocating routine.  The caller still
 * passes the accumulation image (and, optionally, the per-sample buffer) as device memory.
 *   - width*height above REINA_NOALLOC_MAX_PIXELS is rejected with REINA_ERR_INVALID.
 *   - The first call on a device looks up the array's device address (cudaGetSymbolAddress) with that
 *     device current; make that first call before any stream capture.  Under CUDA's default lazy module
 *     loading, that first call (or the first call of any entry point that runs the pass-by-pass
 *     wavefront) is also when the driver loads the library's module on the device and reserves the
 *     array; set CUDA_MODULE_LOADING=EAGER to have it reserved when the context is created instead.
 *   - Every call uses the same array: calls whose work overlaps on the GPU (different streams, or
 *     different host threads) race and corrupt each other's images; serialize them. */
enum { REINA_NOALLOC_MAX_PIXELS = 65536 };
int reina_render_device_noalloc(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* push_consts,
                                const reina_render_options* options, void* d_accum_rgba32f, void* d_samples_rgb32f,
                                void* stream);

/* Batched renders.  No counterpart in the reference, which renders one scene per vkCmdTraceRaysKHR:
 * here many frames — different scenes, resolutions, sample counts, depths and modes — are traced
 * together in shared waves of `wave_paths` path slots, each wave a replayed CUDA graph of the wavefront
 * kernels.  Every job gives the same image (and per-sample colours) as reina_render_device on its own:
 * a job's samples of one pixel are traced and summed in sample order, whatever else shares the waves.
 * options.flags must be 0. */
typedef struct reina_render_job {
    const reina_scene* scene;    /* built scene of this context */
    RtPushConsts push_consts;
    reina_render_options options;
    void* accum_rgba32f;         /* width*height RGBA32F: read when sampleBatch > 0, then written */
    void* samples_rgb32f;        /* optional width*height*spp*3 floats */
} reina_render_job;

/* Host buffers: copies the images in and out; blocks until every job is done. */
int reina_render_batch(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, reina_render_stats* stats);
/* Device buffers (16-byte aligned accumulation images); runs the waves on `stream` and returns when the
 * last one has finished. */
int reina_render_batch_device(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, void* stream,
                              reina_render_stats* stats);

/* ------------------------------------------------------------------------------------------------ */
/* Request server.  No counterpart in the reference, whose run loop renders one scene frame after      */
/* frame (src/Reina.cpp:425-470 driven by src/main.cpp).  A server owns a loop thread that admits      */
/* render requests as they arrive — while device memory within the budget allows — and runs every      */
/* admitted request in shared waves of the batched wavefront; requests join and leave between waves,   */
/* and several waves are in flight at once (the next are packed and running while the last bounces of  */
/* the earlier ones finish).                                                                           */
/* Scenes and kept images stay resident and are evicted least-recently-used when admission needs room */
/* (evicted images are kept in host memory and restored on their next use).  A request's image is the */
/* one reina_render gives for the same scene, push constants and options.                            */
/* ------------------------------------------------------------------------------------------------ */
typedef struct reina_server reina_server;

typedef struct reina_server_options {
    uint64_t memory_budget_bytes; /* device memory for resident scenes, kept images, running requests and
                                   * the path state of the waves in flight (wave_lanes x wave_paths x
                                   * 164 bytes, + 64 MiB of descriptors and slack) (0 = 120e9 bytes) */
    uint32_t max_active_jobs;     /* requests sharing the waves, 1..512 (0 = 512) */
    uint32_t wave_paths;          /* path slots per wave (0 = REINA_SERVER_WAVE_PATHS) */
    uint32_t flags;               /* REINA_BATCH_NO_GRAPHS, and at most one of REINA_SERVER_SHORTEST,
                                   * REINA_SERVER_FIFO, REINA_SERVER_FAIR_SHARE */
    uint32_t wave_lanes;          /* waves in flight, 1..16 (0 = REINA_SERVER_WAVE_LANES) */
    float aging;                  /* REINA_SERVER_SHORTEST: seconds of priority per second waited
                                   * (0 = REINA_SERVER_DEFAULT_AGING; negative = none) */
    uint32_t reserved;
} reina_server_options;
/* Scheduling of the wave slots:
 *   REINA_SERVER_SHORTEST    (the default) the running requests with the least work left first
 *                            (ties: the oldest), each taking all it can use — the shortest-remaining-
 *                            work order.  With aging > 0 the order key is the request's estimated
 *                            remaining time (samples left / the server's measured samples per second)
 *                            minus aging x the time since it was submitted, so that long requests are
 *                            not passed over indefinitely (on the stream below, aging 0 / 0.03 / 0.06 /
 *                            0.12 gives p50 0.21 / 0.22 / 0.34 / 1.04 s and p99 4.9 / 4.0 / 3.2 / 2.5 s
 *                            at the same throughput);
 *   REINA_SERVER_FIFO        the oldest running requests first, each taking all it can use — lower
 *                            latency for the requests at the head, higher for the ones behind them;
 *   REINA_SERVER_FAIR_SHARE  an equal share per running request, leftovers to the oldest.
 * On a Poisson stream of 169 requests (50/s over the 256-scene batched workload's distribution) they
 * give p50 / p99 latency 0.26 / 6.1 s (shortest), 2.3 / 3.6 s (fifo) and 1.2 / 6.9 s (fair share), and
 * 23.2, 22.9 and 20.7 renders/s. */
enum { REINA_SERVER_FIFO = 2, REINA_SERVER_SHORTEST = 4, REINA_SERVER_FAIR_SHARE = 8 };
#define REINA_SERVER_DEFAULT_AGING 0.03f

/* A server runs on its context's GPU; destroying the context destroys its servers first. */
int reina_server_create(reina_ctx* ctx, const reina_server_options* options, reina_server** out_server);
/* Cancels queued and running requests, joins the loop thread, destroys the server's scenes. */
void reina_server_destroy(reina_server* server);

/* Hands a built scene of the server's context to the server, which owns it from now on (do not use or
 * destroy the handle afterwards). */
int reina_server_add_scene(reina_server* server, reina_scene* scene, uint32_t* out_scene_id);

typedef struct reina_request {
    uint32_t scene_id;            /* from reina_server_add_scene */
    uint32_t reserved;
    uint64_t image_key;           /* 0: the image lives only for the request.  Otherwise the finished image
                                   * stays with the server under this key, and a later request with the
                                   * same key, size and sampleBatch > 0 accumulates onto it (progressive
                                   * rendering) without a host round trip. */
    RtPushConsts push_consts;
    reina_render_options options; /* flags must be 0 */
    float* accum_rgba32f;         /* host, width*height RGBA32F: written when the request completes (and
                                   * read at admission when sampleBatch > 0 and image_key is 0); it must
                                   * stay valid until then.  May be NULL when image_key != 0. */
} reina_request;

enum {
    REINA_REQ_QUEUED = 0,
    REINA_REQ_RUNNING = 1,
    REINA_REQ_DONE = 2,
    REINA_REQ_FAILED = 3,
    REINA_REQ_CANCELLED = 4
};

typedef struct reina_request_status {
    uint32_t state;               /* REINA_REQ_* */
    int32_t error;                /* REINA_ERR_* of a failed request */
    double latency_s;             /* submit -> result in the host image (or -> failure / cancellation) */
    double queue_s;               /* submit -> admission */
    char message[160];
} reina_request_status;

/* Queues a request (does not block on the GPU).  REINA_ERR_BUDGET if the request can never fit the
 * budget, even with everything else evicted. */
int reina_server_submit(reina_server* server, const reina_request* request, uint64_t* out_request_id);
int reina_server_poll(reina_server* server, uint64_t request_id, reina_request_status* out_status);
/* Blocks until the request is done, failed or cancelled, or for timeout_s seconds (< 0: no limit). */
int reina_server_wait(reina_server* server, uint64_t request_id, double timeout_s, reina_request_status* out_status);
int reina_server_cancel(reina_server* server, uint64_t request_id);
/* Copies the finished image kept under image_key to the host (accum_rgba32f may be NULL to query the
 * size). */
int reina_server_fetch_image(reina_server* server, uint64_t image_key, float* accum_rgba32f, uint32_t* out_width,
                             uint32_t* out_height);

typedef struct reina_server_stats {
    uint64_t submitted, completed, failed, cancelled, queued, running;
    double latency_p50_s, latency_p99_s, latency_mean_s, latency_max_s;   /* completed requests */
    double uptime_s;
    double busy_s;                /* wall time spent in waves */
    double first_submit_to_last_done_s;
    uint64_t rays, shadow_rays, waves;
    uint64_t scene_uploads, scene_evictions, image_evictions, image_restores;
    uint64_t resident_bytes, peak_resident_bytes, budget_bytes, reserved_bytes;
} reina_server_stats;
int reina_server_get_stats(reina_server* server, reina_server_stats* out_stats);

/* ------------------------------------------------------------------------------------------------ */
/* Post-process — replaces Reina::applyBloom + Reina::applyTonemapping (src/Reina.cpp:472-577):        */
/* blurX (threshold) -> blurY -> combine (shaders/postprocessing/bloom), then exposure and the          */
/* ACES fitted curve to RGBA8 UNORM (shaders/postprocessing/tonemap/tonemapping.comp.glsl:66-84).      */
/* ------------------------------------------------------------------------------------------------ */
/* Host buffers: accum width*height RGBA32F in, rgba8 width*height*4 bytes out; combined_rgba32f
 * (optional) receives the bloomed HDR image before tone mapping. */
int reina_postprocess(reina_ctx* ctx, const float* accum_rgba32f, uint32_t width, uint32_t height,
                      const BloomPushConsts* bloom, const TonemappingPushConsts* tonemap, uint8_t* rgba8,
                      float* combined_rgba32f);

/* Device buffers, enqueued on `stream`. */
int reina_postprocess_device(reina_ctx* ctx, const void* d_accum_rgba32f, uint32_t width, uint32_t height,
                             const BloomPushConsts* bloom, const TonemappingPushConsts* tonemap, void* d_rgba8,
                             void* d_combined_rgba32f, void* stream);

/* ------------------------------------------------------------------------------------------------ */
/* Camera  (src/graphics/Camera.cpp:10-11)                                                           */
/* ------------------------------------------------------------------------------------------------ */
/* inverse(perspective(fovy_radians, aspect, near, far)) and inverse(lookAt(pos, pos + front, up)),
 * column-major, as glm computes them. */
int reina_camera_matrices(const float pos[3], const float front[3], const float up[3], float fovy_radians,
                          float aspect, float z_near, float z_far, float inv_view[16], float inv_proj[16]);

/* ------------------------------------------------------------------------------------------------ */
/* Loaders, run configuration and image output                                                      */
/* ------------------------------------------------------------------------------------------------ */
/* Scene::defineObject(filepath) (src/scene/Scene.h:70; Models::getObjData, src/scene/Models.cpp:117-175):
 * a Wavefront OBJ file as one model — polygons fanned into triangles, one vertex per distinct
 * (position, UV, normal) triple, smooth normals where the file has none, UVs flipped (v -> 1 - v),
 * per-vertex tangent frames from the UVs (zero tangent and bitangent without UVs, as the reference
 * leaves them). */
int reina_scene_define_object_obj(reina_scene* scene, const char* path, uint32_t* out_object_id);

typedef struct reina_gltf_stats {
    uint32_t meshes;
    uint32_t primitives;          /* objects defined (triangle primitives) */
    uint32_t instances;           /* instances added (node x primitive) */
    uint32_t skipped_primitives;  /* non-triangle or empty primitives */
    uint32_t ignored_textures;    /* texture references left out (image missing or not decodable) */
} reina_gltf_stats;
/* gltf::loadScene (src/scene/gltf/gltfloader.cpp:432-456, less the build): adds the default scene of a
 * .gltf or .glb file (buffers embedded, base64 data URIs or files beside it) to an unbuilt scene — one
 * object per triangle primitive, one instance per (node, primitive) with the node's world matrix, the
 * material mapped as gltfloader.cpp:380-412 maps it (Disney; emissive factor x strength when there is
 * no emissive texture; metallic; roughness clamped to [0.1, 0.7]; base colour; cull unless double-sided;
 * KHR_materials_ior; KHR_materials_transmission -> specular transmission, no culling; baseColorTexture
 * -> texture_id, normalTexture -> normal_map_id).  Every image of the file becomes a scene texture in
 * image order (gltfloader.cpp:283-340; never flipped); images that do not decode (formats other than
 * PNG and sequential JPEG) are left out and the references to them counted in ignored_textures.  A primitive without
 * normals fails as in the reference. */
int reina_scene_add_gltf(reina_scene* scene, const char* path, reina_gltf_stats* out_stats);

/* Textures (Scene::defineTexture, src/scene/Scene.cpp:15-25; sampled by the closest-hit shaders through
 * texture_id / normal_map_id / bump_map_id of reina_material).  Texels are 8-bit RGBA, rows top to
 * bottom, row 0 at v = 0; sampling is bilinear at level 0 with REPEAT addressing (the sampler of
 * src/tools/vktools.cpp:765-780 on an R8G8B8A8_UNORM image).  The returned ids count from 0 in
 * definition order; material ids are checked against them at reina_scene_build (REINA_ERR_INVALID).
 *   _rgba8:   raw texels (width*height*4 bytes)
 *   _file:    an image file, rows flipped vertically as the reference loads paths (src/graphics/Image.cpp:14)
 *   _encoded: an image file's bytes in memory, not flipped (src/graphics/Image.cpp:27-33)
 * Image files: PNG (every colour type and bit depth, as stbi_load(..., 4) converts them) and sequential
 * JPEG (baseline / extended Huffman; texels may differ by a few units from stb_image's); other formats
 * fail with REINA_ERR_IO. */
int reina_scene_define_texture_rgba8(reina_scene* scene, const uint8_t* rgba8, uint32_t width, uint32_t height,
                                     uint32_t* out_texture_id);
int reina_scene_define_texture_file(reina_scene* scene, const char* path, uint32_t* out_texture_id);
int reina_scene_define_texture_encoded(reina_scene* scene, const void* data, uint64_t bytes, uint32_t* out_texture_id);
int reina_scene_texture_count(const reina_scene* scene, uint32_t* out_count);
/* Copies texture `texture_id`'s texels out (rgba8 = NULL: size only; else rgba8_capacity >= w*h*4). */
int reina_scene_export_texture(const reina_scene* scene, uint32_t texture_id, uint32_t* out_width,
                               uint32_t* out_height, uint8_t* rgba8, uint64_t rgba8_capacity);

/* Decodes an image file's bytes to RGBA8 (the conversion the texture calls apply).  Pass rgba8 = NULL to
 * receive only the size; otherwise rgba8_capacity must hold width*height*4 bytes. */
int reina_decode_image(const void* data, uint64_t bytes, uint32_t* out_width, uint32_t* out_height, uint8_t* rgba8,
                       uint64_t rgba8_capacity);

/* Number of objects of a scene, and the model data stored for one (the arrays are copied out; pass NULL
 * for any of them, and *_count pointers receive the sizes in elements: vertices, indices, TBNs, UVs). */
int reina_scene_object_count(const reina_scene* scene, uint32_t* out_count);
int reina_scene_export_object(const reina_scene* scene, uint32_t object_id, float* vertices4, uint64_t* vertex_count,
                              uint32_t* indices, uint64_t* index_count, float* tbns9, uint64_t* tbn_count,
                              float* tex_coords2, uint64_t* tex_coord_count);

/* config/config.toml as the reference reads it (src/Reina.cpp:142-156,185,243-245;
 * src/tools/SaveManager.cpp:6-24).  Every key the reference reads is required; defocus_multiplier is
 * divided by 100 as in src/Reina.cpp:150.  At most 64 save points of each kind. */
enum { REINA_CONFIG_MAX_SAVES = 64 };
typedef struct reina_config {
    float focus_dist;
    float defocus_multiplier;
    uint32_t samples_per_pixel;
    uint32_t max_bounces;
    float direct_clamp;
    float indirect_clamp;
    BloomPushConsts bloom;
    TonemappingPushConsts tonemap;
    uint32_t save_on_samples_count;
    uint32_t save_on_times_count;
    int64_t save_on_samples[REINA_CONFIG_MAX_SAVES];
    double save_on_times[REINA_CONFIG_MAX_SAVES];
    /* optional keys of this build, defaulting to the reference's hard-coded values
     * (src/Reina.cpp:54-55,91,138-140): [render] width, height, seed, mode = "reina" | "nee";
     * [scene] path; [camera] pos = [x, y, z], look_at = [x, y, z], fov (degrees) */
    uint32_t width;
    uint32_t height;
    uint32_t seed;
    uint32_t mode;               /* REINA_MODE_REINA or REINA_MODE_NEE_MIS */
    char scene_path[512];        /* "" when absent */
    float camera_pos[3];
    float look_at[3];
    float fov_degrees;
} reina_config;
int reina_config_load(const char* path, reina_config* out_config);

/* SaveManager (src/tools/SaveManager.cpp:26-39): each save point is taken once, the first time the
 * sample count (time in seconds) exceeds it; next() writes "output_<N>spp.png" / "output_<T>sec.png"
 * into name_out (at least 64 bytes), or "" when nothing is due (sample points are checked first; one
 * per call). */
typedef struct reina_save_schedule reina_save_schedule;
int reina_save_schedule_create(const reina_config* config, reina_save_schedule** out_schedule);
void reina_save_schedule_destroy(reina_save_schedule* schedule);
int reina_save_schedule_next(reina_save_schedule* schedule, uint64_t samples, double seconds, char* name_out,
                             size_t name_capacity);

/* Writes an RGBA8 image (width*height*4 bytes, rows top to bottom) as a PNG file (the reference saves
 * the tone-mapped image with stb_image_write, src/Reina.cpp:19-47). */
int reina_write_png(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);

/* Device self-check: evaluates single device shading functions on fixed inputs (case records of 40
 * floats, host buffers; 4 floats out per case) so that a port can pin them against known answers:
 *   REINA_KAT_OFFSET      offsetPositionAlongNormal (closestHitCommon.h.glsl:156-177): p = r[0..2], n = r[3..5]
 *   REINA_KAT_GGX_VNDF    sampleGGXVNDF (brdfDisney.h.glsl:9-40): V = r[0..2], ax = r[6], ay = r[7], RNG
 *                         state = bits of r[8]; out[3] = the RNG state after the two draws (bits)
 *   REINA_KAT_EVAL_DISNEY evalDisney (brdfDisney.h.glsl:656-711): parameters in r[0..18], n r[19..21],
 *                         wi r[22..24], wo r[25..27], TBN columns r[28..36]; out = f, pdf
 *   REINA_KAT_RANDOM      random (shaderCommon.h.glsl:39-45): state = bits of r[0]; out = three draws and
 *                         the state after (bits)
 *   REINA_KAT_OFFSET_DIELECTRIC offsetPositionForDielectric (dielectric.rchit.glsl:14-38): p = r[0..2],
 *                         n = r[3..5], ray direction r[6..8]
 *   REINA_KAT_SAMPLE_DISNEY sampleDisney (brdfDisney.h.glsl:609-654): base r[0..2], anisotropic r[9],
 *                         roughness r[10], clearcoatGloss r[12], metallic r[13], clearcoat r[14],
 *                         specularTransmission r[15], eta r[17], n r[19..21], wi r[22..24], TBN columns
 *                         r[28..36], state = bits of r[37]; out = the direction, the state after (bits)
 *   REINA_KAT_SAMPLE_DISNEY_LOBE the same sample; out = didRefract, choseGlass (0 or 1)
 *   REINA_KAT_DIFFUSE_REFLECTION diffuseReflection (closestHitCommon.h.glsl:215-222): n = r[0..2],
 *                         state = bits of r[8]; out = the direction, the state after (bits)
 *   REINA_KAT_RANDOM_UNIT_VEC randomUnitVec (closestHitCommon.h.glsl:195-205): state = bits of r[8];
 *                         out = the vector, the state after (bits) */
enum {
    REINA_KAT_OFFSET = 0, REINA_KAT_GGX_VNDF = 1, REINA_KAT_EVAL_DISNEY = 2, REINA_KAT_RANDOM = 3,
    REINA_KAT_OFFSET_DIELECTRIC = 4, REINA_KAT_SAMPLE_DISNEY = 5, REINA_KAT_DIFFUSE_REFLECTION = 6,
    REINA_KAT_RANDOM_UNIT_VEC = 7, REINA_KAT_SAMPLE_DISNEY_LOBE = 15
};
int reina_device_kat(reina_ctx* ctx, int kind, const float* records, uint64_t count, float* out);

/* ------------------------------------------------------------------------------------------------ */
/* Autotuner                                                                                          */
/* ------------------------------------------------------------------------------------------------ */
/* Autotuner (no counterpart in the reference).  Each reina_autotune_* call times candidate
 * configurations on the caller's own workload — the traversal launch form, block size and stack depth
 * (every variant in reina_tuning), and for batched renders also the wave size — and stores the fastest
 * in the context's cache under (kind, floor(log2(triangles)), floor(log2(work size))), where the work
 * size is the ray count, the pixel count, or the batch's total samples.  With REINA_AUTOTUNE_CACHED,
 * ray casts, renders and batched renders whose key is in the cache run with the cached configuration
 * instead of the context's tuning.  Results never depend on the configuration. */
enum {
    REINA_TUNE_RAYCAST_CLOSEST = 0,
    REINA_TUNE_RAYCAST_ANY = 1,
    REINA_TUNE_RENDER = 2,
    REINA_TUNE_BATCH = 3
};
enum { REINA_AUTOTUNE_OFF = 0, REINA_AUTOTUNE_CACHED = 1 };

typedef struct reina_tune_result {
    reina_tuning best;            /* the fastest candidate (refill, trace_block, trace_stack; wave_paths
                                   * for REINA_TUNE_BATCH) */
    double best_ms;               /* its time per call (median of the timed calls) */
    double default_ms;            /* the default configuration's time per call */
    uint32_t candidates;          /* configurations timed */
    uint32_t kind;                /* REINA_TUNE_* */
    uint32_t tri_bucket;          /* cache key parts */
    uint32_t size_bucket;
} reina_tune_result;

/* Times the ray cast of `count` device rays into `d_hits` (flags as reina_raycast_device) on `stream`
 * for every candidate; blocks until done.  The hit buffer holds the (configuration-independent) hits
 * afterwards. */
int reina_autotune_raycast(reina_ctx* ctx, const reina_scene* scene, const void* d_rays, uint64_t count,
                           void* d_hits, uint32_t flags, void* stream, reina_tune_result* out_result);
/* Times one-sample frames of the render (scratch image; the caller's images are not touched). */
int reina_autotune_render(reina_ctx* ctx, const reina_scene* scene, const RtPushConsts* push_consts,
                          const reina_render_options* options, reina_tune_result* out_result);
/* Times a batched render of (up to 32 of) the jobs at no more than 2 samples per pixel, into scratch
 * images. */
int reina_autotune_batch(reina_ctx* ctx, const reina_render_job* jobs, uint32_t count, reina_tune_result* out_result);
int reina_autotune_set_mode(reina_ctx* ctx, uint32_t mode);
/* The cached configuration for a workload, if any (*out_found = 0 when there is none). */
int reina_autotune_lookup(reina_ctx* ctx, uint32_t kind, uint64_t triangles, uint64_t work_size,
                          reina_tuning* out_tuning, int32_t* out_found);
/* Writes / merges the cache as text, one "kind tri_bucket size_bucket refill block stack wave_paths
 * best_ms default_ms" line per entry. */
int reina_autotune_save(reina_ctx* ctx, const char* path);
int reina_autotune_load(reina_ctx* ctx, const char* path);

/* ------------------------------------------------------------------------------------------------ */
/* Synthetic workloads (seeded, deterministic)                                                        */
/* ------------------------------------------------------------------------------------------------ */
/* Vertex and triangle counts of a level-`level` subdivided icosphere: 10*4^L + 2 and 20*4^L. */
int reina_icosphere_counts(uint32_t level, uint64_t* out_vertices, uint64_t* out_triangles);

/* Level-`level` icosphere of radius 1, each vertex displaced radially to r = 1 + amplitude * n(p)
 * with n a 3-octave value noise in [-1, 1] keyed by `seed`.  vertices: 4 floats per vertex (w = 1);
 * normals (optional, 3 floats per vertex): normalized vertex positions before displacement. */
int reina_gen_icosphere(uint32_t level, float amplitude, uint64_t seed, float* vertices,
                        uint32_t* indices, float* normals);

/* Class-I geodesic sphere of frequency n (each icosahedron face cut into an n x n triangular grid):
 * 10*n^2 + 2 vertices and 20*n^2 triangles, so triangle counts between icosphere levels are reachable.
 * Grid points are placed on the flat face and then projected (the icosphere projects at every halving,
 * so frequency 2^L is not the level-L icosphere).  Displacement, vertex and normal layout as
 * reina_gen_icosphere. */
int reina_geodesic_counts(uint32_t frequency, uint64_t* out_vertices, uint64_t* out_triangles);
int reina_gen_geodesic(uint32_t frequency, float amplitude, uint64_t seed, float* vertices, uint32_t* indices,
                       float* normals);

/* The two ray sets of the ray-cast workload: `n_camera` pinhole rays through pixel centres of a
 * width x height image from `cam_pos` looking at `cam_target` (fovy degrees), followed by `n_random`
 * rays with origins uniform in `box_min..box_max` and directions uniform on the sphere (SplitMix64
 * keyed by `seed`).  tmin = 0, tmax = 1e4.  Returns n_camera = width*height rays first. */
int reina_gen_raycast_rays(uint32_t width, uint32_t height, const float cam_pos[3], const float cam_target[3],
                           float fovy_degrees, uint64_t n_random, const float box_min[3],
                           const float box_max[3], uint64_t seed, reina_ray* rays_out);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* REINA_C_H */
