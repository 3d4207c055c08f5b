// The reference's run configuration (config/config.toml, read at src/Reina.cpp:51,142-156,185,243-245
// and src/tools/SaveManager.cpp:6-24), its PNG save schedule (SaveManager::shouldSave,
// src/tools/SaveManager.cpp:26-39) and a PNG writer for the tone-mapped image.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace rt {

// A TOML subset: [table] and [a.b] headers, key = value with integers, floats, booleans, basic strings
// and one-line arrays of those, '#' comments.  Values are addressed by dotted path ("sampling.max_bounces").
struct TomlValue {
    enum Kind { Int, Float, Bool, String, Array } kind = Int;
    int64_t i = 0;
    double f = 0.0;
    bool b = false;
    std::string s;
    std::vector<TomlValue> arr;
    double as_double() const { return kind == Int ? (double)i : f; }
};
std::map<std::string, TomlValue> parse_toml(const std::string& text, const std::string& name);

struct RunConfig {
    float focus_dist = 1.0f;
    float defocus_multiplier = 0.0f;   // already divided by 100, as src/Reina.cpp:150 does
    uint32_t samples_per_pixel = 1;
    uint32_t max_bounces = 8;
    float direct_clamp = 100.0f;
    float indirect_clamp = 10.0f;
    std::vector<int64_t> save_on_samples;
    std::vector<double> save_on_times;
    float bloom_radius = 5.0f, bloom_threshold = 1.0f, bloom_intensity = 0.05f;
    float exposure = 0.0f;
    // Optional keys of this build (the reference hard-codes these, src/Reina.cpp:54-55,91,138-140; the
    // defaults are its values): [render] width, height, seed, mode ("reina" | "nee"); [scene] path;
    // [camera] pos, look_at (3-element arrays), fov (degrees).
    uint32_t width = 1080, height = 1350, seed = 1;
    uint32_t mode = 0;   // 0 reina, 1 NEE + MIS
    std::string scene_path;
    float camera_pos[3] = {-1.6899f, 0.317017f, 1.6386f};
    float look_at[3] = {0.0f, 0.962f, 0.0f};
    float fov_degrees = 25.0f;
};
// Every key the reference reads is required (the reference's .value() throws when one is missing); the
// optional keys above keep their defaults when absent.
RunConfig load_config(const std::string& path);
RunConfig config_from_toml(const std::string& text, const std::string& name);

// SaveManager: pending sample counts and times, each consumed in ascending order once exceeded
// (strictly).  next() returns the file name to save now ("" if none): "output_<N>spp.png" or
// "output_<int(T)>sec.png"; sample thresholds are checked first and one save is returned per call.
class SaveSchedule {
public:
    SaveSchedule(std::vector<int64_t> samples, std::vector<double> times);
    std::string next(uint64_t samples, double seconds);
    bool empty() const { return samples_.empty() && times_.empty(); }

private:
    std::vector<int64_t> samples_;   // descending
    std::vector<double> times_;      // descending
};

// RGBA8 PNG (8-bit, colour type 6, no interlace) with stored deflate blocks.
void write_png(const std::string& path, const uint8_t* rgba, uint32_t width, uint32_t height);
std::vector<uint8_t> encode_png(const uint8_t* rgba, uint32_t width, uint32_t height);

}  // namespace rt
