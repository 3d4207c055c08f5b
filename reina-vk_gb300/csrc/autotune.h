// Autotuner cache: the fastest launch configuration per (workload kind, scene-size bucket, work-size
// bucket), filled by timing candidate configurations on a caller's workload, saved to and loaded from a
// small text file, and looked up by the ray-cast, render and batched-render entry points.
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "kernels.h"

namespace rt {

enum TuneKind : uint32_t { kTuneRaycastClosest = 0, kTuneRaycastAny = 1, kTuneRender = 2, kTuneBatch = 3 };

struct TuneEntry {
    TraceConfig trace;
    uint32_t wave_paths = 0;      // batched renders only (0 = default)
    double best_ms = 0.0;
    double default_ms = 0.0;
};

// floor(log2(max(x, 1))): workloads within a factor of two share an entry.
uint32_t tune_bucket(uint64_t x);

class TuneCache {
public:
    void put(uint32_t kind, uint32_t tri_bucket, uint32_t size_bucket, const TuneEntry& e);
    bool get(uint32_t kind, uint32_t tri_bucket, uint32_t size_bucket, TuneEntry* out) const;
    size_t size() const;
    // Text format, one entry per line:
    //   kind tri_bucket size_bucket refill block stack wave_paths best_ms default_ms [order]
    // (order: 0 input ray order, the default when absent; 1 coherence order)
    // Lines starting with '#' are comments.  load() merges into the cache (later lines win).
    void save(const std::string& path) const;
    void load(const std::string& path);

private:
    mutable std::mutex mu_;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t>, TuneEntry> map_;
};

// Candidate traversal configurations: the grid form in every block size x stack depth, and (for ray
// casts) the persistent form at two refill thresholds.
std::vector<TraceConfig> trace_candidates(bool with_order);

}  // namespace rt
