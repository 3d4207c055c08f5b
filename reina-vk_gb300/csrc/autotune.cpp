// Autotuner cache (see autotune.h).
#include "autotune.h"

#include <fstream>
#include <sstream>

#include "errors.h"

namespace rt {

uint32_t tune_bucket(uint64_t x) {
    uint32_t b = 0;
    while (x > 1) {
        x >>= 1;
        ++b;
    }
    return b;
}

void TuneCache::put(uint32_t kind, uint32_t tri_bucket, uint32_t size_bucket, const TuneEntry& e) {
    std::lock_guard<std::mutex> lk(mu_);
    map_[std::make_tuple(kind, tri_bucket, size_bucket)] = e;
}

bool TuneCache::get(uint32_t kind, uint32_t tri_bucket, uint32_t size_bucket, TuneEntry* out) const {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = map_.find(std::make_tuple(kind, tri_bucket, size_bucket));
    if (it == map_.end()) return false;
    if (out) *out = it->second;
    return true;
}

size_t TuneCache::size() const {
    std::lock_guard<std::mutex> lk(mu_);
    return map_.size();
}

void TuneCache::save(const std::string& path) const {
    std::lock_guard<std::mutex> lk(mu_);
    std::ofstream f(path);
    if (!f) fail(REINA_ERR_IO, "cannot write autotune cache: " + path);
    f << "# kind tri_bucket size_bucket refill block stack wave_paths best_ms default_ms order\n";
    f.precision(9);
    for (const auto& [k, e] : map_) {
        f << std::get<0>(k) << ' ' << std::get<1>(k) << ' ' << std::get<2>(k) << ' ' << e.trace.refill << ' '
          << e.trace.block << ' ' << e.trace.stack << ' ' << e.wave_paths << ' ' << e.best_ms << ' ' << e.default_ms
          << ' ' << e.trace.sort << '\n';
    }
    if (!f) fail(REINA_ERR_IO, "cannot write autotune cache: " + path);
}

void TuneCache::load(const std::string& path) {
    std::ifstream f(path);
    if (!f) fail(REINA_ERR_IO, "cannot read autotune cache: " + path);
    std::map<std::tuple<uint32_t, uint32_t, uint32_t>, TuneEntry> add;
    std::string line;
    int lineno = 0;
    while (std::getline(f, line)) {
        ++lineno;
        const size_t first = line.find_first_not_of(" \t\r");
        if (first == std::string::npos || line[first] == '#') continue;
        std::istringstream is(line);
        uint32_t kind, tb, sb, wave;
        TuneEntry e;
        if (!(is >> kind >> tb >> sb >> e.trace.refill >> e.trace.block >> e.trace.stack >> wave >> e.best_ms >>
              e.default_ms))
            fail(REINA_ERR_IO, path + ":" + std::to_string(lineno) + ": malformed autotune entry");
        uint32_t order = 0;   // optional tenth field: 0 input ray order (default), 1 coherence order
        if (is >> order) {
            if (order > 1) fail(REINA_ERR_IO, path + ":" + std::to_string(lineno) + ": invalid ray order");
        } else if (!is.eof()) {
            fail(REINA_ERR_IO, path + ":" + std::to_string(lineno) + ": malformed autotune entry");
        }
        e.trace.sort = (int)order;
        std::string rest;
        is.clear();
        if (is >> rest) fail(REINA_ERR_IO, path + ":" + std::to_string(lineno) + ": trailing text in autotune entry");
        if (kind > kTuneBatch || !valid_trace_config(e.trace) || wave > (1u << 26))
            fail(REINA_ERR_IO, path + ":" + std::to_string(lineno) + ": invalid autotune entry");
        e.wave_paths = wave;
        add[std::make_tuple(kind, tb, sb)] = e;
    }
    std::lock_guard<std::mutex> lk(mu_);
    for (const auto& [k, e] : add) map_[k] = e;
}

std::vector<TraceConfig> trace_candidates(bool with_order) {
    std::vector<TraceConfig> out;
    for (int block : {64, 128, 256})
        for (int stack : {8, 12, 16}) {
            TraceConfig c;
            c.block = block;
            c.stack = stack;
            c.refill = 0;
            out.push_back(c);
        }
    if (with_order) {   // ray casts: also coherence order, in the default block size and stack depth
        TraceConfig c;
        c.refill = 0;
        c.sort = 1;
        out.push_back(c);
    }
    for (int refill : {4, 8, 16}) {   // the cooperative form
        TraceConfig c;
        c.refill = refill;
        out.push_back(c);
    }
    return out;
}

}  // namespace rt
