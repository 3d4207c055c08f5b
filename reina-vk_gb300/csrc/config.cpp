// Run configuration, save schedule and PNG writer (see config.h).
#include "config.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <sstream>

#include "errors.h"

namespace rt {

namespace {

std::string trim(const std::string& s) {
    const size_t a = s.find_first_not_of(" \t\r");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r");
    return s.substr(a, b - a + 1);
}

// Removes a '#' comment that is not inside a string.
std::string strip_comment(const std::string& s) {
    bool in_str = false;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] == '"' && (i == 0 || s[i - 1] != '\\')) in_str = !in_str;
        if (s[i] == '#' && !in_str) return s.substr(0, i);
    }
    return s;
}

struct ValueParser {
    const std::string& s;
    size_t p = 0;
    std::string where;

    [[noreturn]] void bad(const std::string& what) const { fail(REINA_ERR_IO, where + ": " + what); }
    void ws() {
        while (p < s.size() && (s[p] == ' ' || s[p] == '\t')) ++p;
    }
    TomlValue value() {
        ws();
        if (p >= s.size()) bad("missing value");
        TomlValue v;
        if (s[p] == '[') {
            v.kind = TomlValue::Array;
            ++p;
            ws();
            if (p < s.size() && s[p] == ']') {
                ++p;
                return v;
            }
            while (true) {
                v.arr.push_back(value());
                ws();
                if (p < s.size() && s[p] == ',') {
                    ++p;
                    ws();
                    if (p < s.size() && s[p] == ']') { ++p; break; }   // trailing comma
                    continue;
                }
                if (p < s.size() && s[p] == ']') { ++p; break; }
                bad("expected ',' or ']' in array");
            }
            return v;
        }
        if (s[p] == '"') {
            v.kind = TomlValue::String;
            ++p;
            while (true) {
                if (p >= s.size()) bad("unterminated string");
                const char c = s[p++];
                if (c == '"') break;
                if (c == '\\' && p < s.size()) {
                    const char e = s[p++];
                    v.s += e == 'n' ? '\n' : e == 't' ? '\t' : e;
                } else {
                    v.s += c;
                }
            }
            return v;
        }
        size_t q = p;
        while (q < s.size() && s[q] != ',' && s[q] != ']' && s[q] != ' ' && s[q] != '\t') ++q;
        std::string tok = s.substr(p, q - p);
        p = q;
        if (tok == "true" || tok == "false") {
            v.kind = TomlValue::Bool;
            v.b = tok == "true";
            return v;
        }
        tok.erase(std::remove(tok.begin(), tok.end(), '_'), tok.end());
        char* stop = nullptr;
        const bool is_float = tok.find_first_of(".eE") != std::string::npos || tok == "inf" || tok == "+inf" ||
                              tok == "-inf" || tok == "nan";
        if (is_float) {
            v.kind = TomlValue::Float;
            v.f = std::strtod(tok.c_str(), &stop);
        } else {
            v.kind = TomlValue::Int;
            v.i = std::strtoll(tok.c_str(), &stop, 10);
        }
        if (tok.empty() || stop != tok.c_str() + tok.size()) bad("malformed value '" + tok + "'");
        return v;
    }
};

}  // namespace

std::map<std::string, TomlValue> parse_toml(const std::string& text, const std::string& name) {
    std::map<std::string, TomlValue> out;
    std::istringstream in(text);
    std::string line, table;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        const std::string where = name + ":" + std::to_string(lineno);
        const std::string l = trim(strip_comment(line));
        if (l.empty()) continue;
        if (l[0] == '[') {
            if (l.back() != ']' || l.size() < 3 || l[1] == '[') fail(REINA_ERR_IO, where + ": malformed table header");
            table = trim(l.substr(1, l.size() - 2));
            continue;
        }
        const size_t eq = l.find('=');
        if (eq == std::string::npos) fail(REINA_ERR_IO, where + ": expected key = value");
        const std::string key = trim(l.substr(0, eq));
        if (key.empty()) fail(REINA_ERR_IO, where + ": empty key");
        const std::string rest = l.substr(eq + 1);
        ValueParser vp{rest, 0, where};
        TomlValue v = vp.value();
        vp.ws();
        if (vp.p != rest.size()) fail(REINA_ERR_IO, where + ": trailing characters after value");
        const std::string path = table.empty() ? key : table + "." + key;
        if (out.count(path)) fail(REINA_ERR_IO, where + ": duplicate key " + path);
        out[path] = v;
    }
    return out;
}

RunConfig config_from_toml(const std::string& text, const std::string& name) {
    const auto t = parse_toml(text, name);
    auto need = [&](const std::string& k) -> const TomlValue& {
        auto it = t.find(k);
        if (it == t.end()) fail(REINA_ERR_IO, name + ": missing " + k);
        return it->second;
    };
    auto num = [&](const std::string& k) {
        const TomlValue& v = need(k);
        if (v.kind != TomlValue::Int && v.kind != TomlValue::Float) fail(REINA_ERR_IO, name + ": " + k + " must be a number");
        return v.as_double();
    };
    auto uint = [&](const std::string& k) {
        const TomlValue& v = need(k);
        if (v.kind != TomlValue::Int || v.i < 0 || v.i > 0xFFFFFFFFll)
            fail(REINA_ERR_IO, name + ": " + k + " must be a non-negative integer");
        return (uint32_t)v.i;
    };
    RunConfig c;
    c.focus_dist = (float)num("camera.dof.focus_dist");
    c.defocus_multiplier = (float)num("camera.dof.defocus_multiplier") / 100.0f;
    c.samples_per_pixel = uint("sampling.samples_per_pixel");
    c.max_bounces = uint("sampling.max_bounces");
    c.direct_clamp = (float)num("sampling.direct_clamp");
    c.indirect_clamp = (float)num("sampling.indirect_clamp");
    const TomlValue& ss = need("saving.save_on_samples");
    const TomlValue& st = need("saving.save_on_times");
    if (ss.kind != TomlValue::Array || st.kind != TomlValue::Array) fail(REINA_ERR_IO, name + ": saving lists must be arrays");
    for (const TomlValue& v : ss.arr) {
        if (v.kind != TomlValue::Int) fail(REINA_ERR_IO, name + ": save_on_samples must hold integers");
        c.save_on_samples.push_back(v.i);
    }
    for (const TomlValue& v : st.arr) {
        if (v.kind != TomlValue::Int && v.kind != TomlValue::Float) fail(REINA_ERR_IO, name + ": save_on_times must hold numbers");
        c.save_on_times.push_back(v.as_double());
    }
    c.bloom_radius = (float)num("postprocessing.bloom.radius");
    c.bloom_threshold = (float)num("postprocessing.bloom.threshold");
    c.bloom_intensity = (float)num("postprocessing.bloom.intensity");
    c.exposure = (float)num("postprocessing.tonemap.exposure");
    // optional keys
    auto has = [&](const std::string& k) { return t.find(k) != t.end(); };
    if (has("render.width")) c.width = uint("render.width");
    if (has("render.height")) c.height = uint("render.height");
    if (has("render.seed")) c.seed = uint("render.seed");
    if (has("render.mode")) {
        const TomlValue& v = need("render.mode");
        if (v.kind != TomlValue::String || (v.s != "reina" && v.s != "nee")) fail(REINA_ERR_IO, name + ": render.mode is \"reina\" or \"nee\"");
        c.mode = v.s == "nee" ? 1u : 0u;
    }
    if (has("scene.path")) {
        const TomlValue& v = need("scene.path");
        if (v.kind != TomlValue::String) fail(REINA_ERR_IO, name + ": scene.path must be a string");
        c.scene_path = v.s;
    }
    auto vec3 = [&](const std::string& k, float out[3]) {
        const TomlValue& v = need(k);
        if (v.kind != TomlValue::Array || v.arr.size() != 3) fail(REINA_ERR_IO, name + ": " + k + " must be an array of 3 numbers");
        for (int i = 0; i < 3; ++i) {
            if (v.arr[(size_t)i].kind != TomlValue::Int && v.arr[(size_t)i].kind != TomlValue::Float)
                fail(REINA_ERR_IO, name + ": " + k + " must be an array of 3 numbers");
            out[i] = (float)v.arr[(size_t)i].as_double();
        }
    };
    if (has("camera.pos")) vec3("camera.pos", c.camera_pos);
    if (has("camera.look_at")) vec3("camera.look_at", c.look_at);
    if (has("camera.fov")) c.fov_degrees = (float)num("camera.fov");
    if (c.width == 0 || c.height == 0) fail(REINA_ERR_IO, name + ": render.width and render.height must be positive");
    return c;
}

RunConfig load_config(const std::string& path) {
    std::ifstream f(path);
    if (!f) fail(REINA_ERR_IO, "cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return config_from_toml(ss.str(), path);
}

SaveSchedule::SaveSchedule(std::vector<int64_t> samples, std::vector<double> times)
    : samples_(std::move(samples)), times_(std::move(times)) {
    std::sort(samples_.begin(), samples_.end(), std::greater<>());
    std::sort(times_.begin(), times_.end(), std::greater<>());
}

std::string SaveSchedule::next(uint64_t samples, double seconds) {
    if (!samples_.empty() && samples_.back() < (int64_t)samples) {
        const int64_t n = samples_.back();
        samples_.pop_back();
        return "output_" + std::to_string(n) + "spp.png";
    }
    if (!times_.empty() && times_.back() < seconds) {
        const double t = times_.back();
        times_.pop_back();
        return "output_" + std::to_string((int)t) + "sec.png";
    }
    return "";
}

// ------------------------------------------------------------------------------------------------
// PNG (ISO/IEC 15948): signature, IHDR, one IDAT holding a zlib stream of stored deflate blocks, IEND.

namespace {

uint32_t crc32_update(uint32_t crc, const uint8_t* d, size_t n) {
    static const std::vector<uint32_t> table = [] {
        std::vector<uint32_t> t(256);
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ d[i]) & 0xFF] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<uint8_t>& o, uint32_t v) {
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
    put_be32(out, (uint32_t)data.size());
    const size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    const uint32_t crc = crc32_update(0xFFFFFFFFu, out.data() + start, out.size() - start) ^ 0xFFFFFFFFu;
    put_be32(out, crc);
}

}  // namespace

std::vector<uint8_t> encode_png(const uint8_t* rgba, uint32_t w, uint32_t h) {
    if (w == 0 || h == 0) fail(REINA_ERR_INVALID, "PNG: empty image");
    std::vector<uint8_t> raw;   // filter byte 0 + row
    raw.reserve((size_t)h * (4ull * w + 1));
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba + 4ull * w * y, rgba + 4ull * w * (y + 1));
    }
    std::vector<uint8_t> z = {0x78, 0x01};   // zlib header: deflate, 32K window, no preset dictionary
    size_t off = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
        off += n;
    } while (off < raw.size());
    uint32_t a = 1, b = 0;   // Adler-32
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    chunk(out, "IHDR", ihdr);
    chunk(out, "IDAT", z);
    chunk(out, "IEND", {});
    return out;
}

void write_png(const std::string& path, const uint8_t* rgba, uint32_t w, uint32_t h) {
    const std::vector<uint8_t> png = encode_png(rgba, w, h);
    std::ofstream f(path, std::ios::binary);
    if (!f) fail(REINA_ERR_IO, "cannot write " + path);
    f.write(reinterpret_cast<const char*>(png.data()), (std::streamsize)png.size());
    if (!f) fail(REINA_ERR_IO, "cannot write " + path);
}

}  // namespace rt
