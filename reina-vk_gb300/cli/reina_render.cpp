// reina_render: the reference's run loop (src/Reina.cpp:296-392) without a window.  It reads
// config/config.toml, loads an OBJ model or a glTF scene, renders frame after frame with the GB300 trace
// path (sampleBatch = frame, running mean in the accumulation image), bloom + tone-maps each frame, and
// writes PNGs when the SaveManager schedule says so, plus the final frame.  Uses only the C ABI.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "reina/reina_c.h"

namespace {

[[noreturn]] void die(const std::string& what) {
    std::fprintf(stderr, "reina_render: %s\n", what.c_str());
    std::exit(1);
}

void check(int status, const char* what) {
    if (status != REINA_OK) die(std::string(what) + ": " + reina_last_error());
}

bool parse3(const char* s, float v[3]) { return std::sscanf(s, "%f,%f,%f", &v[0], &v[1], &v[2]) == 3; }

bool ends_with(const std::string& s, const std::string& e) {
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

void usage() {
    std::printf(
        "usage: reina_render --config config.toml [--scene file.{glb,gltf,obj}] [options]\n"
        "  (defaults from the config's optional [render] width/height/seed/mode, [scene] path and\n"
        "   [camera] pos/look_at/fov keys, else the reference's hard-coded values)\n"
        "  --width W --height H        image size (default 1080 x 1350)\n"
        "  --camera x,y,z              camera position (default -1.6899,0.317017,1.6386)\n"
        "  --look-at x,y,z             target (default 0,0.962,0)\n"
        "  --fov DEG                   vertical field of view (default 25)\n"
        "  --frames N | --seconds T    stop after N frames (default 16) or T seconds\n"
        "  --out DIR                   output directory (default .)\n"
        "  --mode reina|nee            integrator (default reina: the reference's, NEE off)\n"
        "  --seed S  --device D  --env sky|r,g,b  --allow-no-emissive\n");
}

}  // namespace

int main(int argc, char** argv) {
    std::string config_path, scene_path, out_dir = ".", env = "sky";
    uint32_t W = 0, H = 0, frames = 16, seed = 0, mode = 0;
    double seconds = 0.0;
    int device = 0;
    bool allow_no_emissive = false, set_cam = false, set_target = false, set_mode = false, set_seed = false;
    float cam[3], target[3], fov = 0.0f;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&]() -> const char* {
            if (i + 1 >= argc) die("missing value for " + a);
            return argv[++i];
        };
        if (a == "--config") config_path = val();
        else if (a == "--scene") scene_path = val();
        else if (a == "--width") W = (uint32_t)std::atoi(val());
        else if (a == "--height") H = (uint32_t)std::atoi(val());
        else if (a == "--camera") { if (!parse3(val(), cam)) die("--camera wants x,y,z"); set_cam = true; }
        else if (a == "--look-at") { if (!parse3(val(), target)) die("--look-at wants x,y,z"); set_target = true; }
        else if (a == "--fov") fov = (float)std::atof(val());
        else if (a == "--frames") frames = (uint32_t)std::atoi(val());
        else if (a == "--seconds") seconds = std::atof(val());
        else if (a == "--out") out_dir = val();
        else if (a == "--mode") {
            const std::string m = val();
            if (m == "reina") mode = REINA_MODE_REINA;
            else if (m == "nee") mode = REINA_MODE_NEE_MIS;
            else die("--mode is reina or nee");
            set_mode = true;
        } else if (a == "--seed") { seed = (uint32_t)std::atoi(val()); set_seed = true; }
        else if (a == "--device") device = std::atoi(val());
        else if (a == "--env") env = val();
        else if (a == "--allow-no-emissive") allow_no_emissive = true;
        else if (a == "--help" || a == "-h") { usage(); return 0; }
        else die("unknown option " + a);
    }
    if (config_path.empty()) { usage(); return 2; }
    // the config's optional [render] / [scene] / [camera] keys are the defaults; options override them
    reina_config cfg;
    check(reina_config_load(config_path.c_str(), &cfg), "config");
    if (scene_path.empty()) scene_path = cfg.scene_path;
    if (scene_path.empty()) { usage(); return 2; }
    if (W == 0) W = cfg.width;
    if (H == 0) H = cfg.height;
    if (!set_seed) seed = cfg.seed;
    if (!set_mode) mode = cfg.mode;
    if (fov == 0.0f) fov = cfg.fov_degrees;
    for (int k = 0; k < 3; ++k) {
        if (!set_cam) cam[k] = cfg.camera_pos[k];
        if (!set_target) target[k] = cfg.look_at[k];
    }
    if (W == 0 || H == 0) die("image size must be positive");
    reina_ctx* ctx = nullptr;
    reina_ctx_options co{device, 0};
    check(reina_ctx_create(&co, &ctx), "context");
    reina_scene* scene = nullptr;
    check(reina_scene_create(ctx, &scene), "scene");
    if (ends_with(scene_path, ".obj")) {
        // the reference's commented-out OBJ set-up uses explicit materials; a plain Disney surface here
        reina_material m;
        std::memset(&m, 0, sizeof(m));
        m.material_idx = 3;
        m.texture_id = m.normal_map_id = m.bump_map_id = -1;
        for (int k = 0; k < 3; ++k) { m.albedo[k] = 0.8f; m.sheen_tint[k] = 1.0f; m.specular_tint[k] = 1.0f; }
        m.roughness = 0.5f;
        m.ior = 1.5f;
        m.interp_normals = 1;
        uint32_t obj = 0;
        check(reina_scene_define_object_obj(scene, scene_path.c_str(), &obj), "OBJ");
        const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        check(reina_scene_add_instance(scene, obj, I, &m), "instance");
    } else {
        reina_gltf_stats gs;
        check(reina_scene_add_gltf(scene, scene_path.c_str(), &gs), "glTF");
        std::printf("glTF: %u meshes, %u primitives, %u instances (%u textures ignored)\n", gs.meshes, gs.primitives,
                    gs.instances, gs.ignored_textures);
    }
    check(reina_scene_build(scene, allow_no_emissive ? 0 : 1), "build");
    reina_scene_stats ss;
    check(reina_scene_get_stats(scene, &ss), "stats");
    std::printf("scene: %llu triangles, %llu BVH8 nodes, built in %.2f s\n", (unsigned long long)ss.triangle_count,
                (unsigned long long)ss.node_count, ss.build_seconds);

    float front[3] = {target[0] - cam[0], target[1] - cam[1], target[2] - cam[2]};
    const float up[3] = {0.0f, 1.0f, 0.0f};
    RtPushConsts pc;
    std::memset(&pc, 0, sizeof(pc));
    const float fovy = (float)((double)fov * 3.14159265358979323846 / 180.0);
    check(reina_camera_matrices(cam, front, up, fovy, (float)W / (float)H, 0.1f, 100.0f, pc.invView, pc.invProjection),
          "camera");
    pc.totalEmissiveWeight = reina_scene_emissive_weight(scene);
    pc.focusDist = cfg.focus_dist;
    pc.defocusMultiplier = cfg.defocus_multiplier;
    pc.directClamp = cfg.direct_clamp;
    pc.indirectClamp = cfg.indirect_clamp;
    pc.samplesPerPixel = cfg.samples_per_pixel;
    pc.maxBounces = cfg.max_bounces;
    reina_render_options ro;
    std::memset(&ro, 0, sizeof(ro));
    ro.width = W;
    ro.height = H;
    ro.mode = mode;
    ro.seed = seed;
    if (env != "sky") {
        ro.env_mode = REINA_ENV_CONSTANT;
        if (!parse3(env.c_str(), ro.env_color)) die("--env is sky or r,g,b");
    }

    std::vector<float> accum(4ull * W * H, 0.0f);
    std::vector<uint8_t> rgba(4ull * W * H);
    reina_save_schedule* sched = nullptr;
    check(reina_save_schedule_create(&cfg, &sched), "save schedule");
    const auto t0 = std::chrono::steady_clock::now();
    uint64_t samples = 0;
    uint32_t frame = 0;
    char name[128];
    auto save = [&](const std::string& file) {
        check(reina_postprocess(ctx, accum.data(), W, H, &cfg.bloom, &cfg.tonemap, rgba.data(), nullptr), "post-process");
        const std::string path = out_dir + "/" + file;
        check(reina_write_png(path.c_str(), rgba.data(), W, H), "PNG");
        std::printf("saved %s\n", path.c_str());
    };
    for (;; ++frame) {
        const double age = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (seconds > 0.0 ? age >= seconds : frame >= frames) break;
        pc.sampleBatch = frame;
        reina_render_stats st;
        check(reina_render(ctx, scene, &pc, &ro, accum.data(), nullptr, &st), "render");
        // the reference asks the SaveManager with the samples of the frames before this one
        check(reina_save_schedule_next(sched, samples, age, name, sizeof(name)), "save schedule");
        if (name[0]) save(name);
        samples += pc.samplesPerPixel;
        std::printf("frame %u: %.1f ms, %.3g segments/s, %llu samples per pixel\n", frame, st.seconds * 1e3,
                    (double)st.rays / st.seconds, (unsigned long long)samples);
    }
    save("output_final.png");
    reina_save_schedule_destroy(sched);
    reina_scene_destroy(scene);
    reina_ctx_destroy(ctx);
    return 0;
}
