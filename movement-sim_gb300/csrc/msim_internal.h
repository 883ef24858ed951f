// Internal declarations shared by the C ABI, the kernels and the host code.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "msim.h"

namespace msim {

// NVTX range over a host scope (the per-tick phases show up by name in Nsight
// timelines; with no tool attached a push/pop is a pointer check).  The reference's
// counterpart is its RenderDoc capture around one tick (Simulator.cpp:403-450).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Thread-local error text behind msim_last_error().
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

// Every device allocation of the library goes through here: cudaMalloc, or a
// failure injected by msim_debug_fail_device_alloc.  True on success.
bool device_malloc(void** p, size_t bytes);

// Owned map (JSON loader, lattice generator).
struct MapData {
    std::vector<float> road_pos;      // 4 per road
    std::vector<uint32_t> road_conn;  // 4 per road
    std::vector<uint32_t> connections;
    float width = 0.f;
    float height = 0.f;
    uint32_t skipped_zero_length = 0;
};

int load_map_json(const char* path, MapData& out);
int write_map_json(const msim_map& map, const char* path);
int generate_lattice(uint32_t side, uint64_t seed, float spacing, float jitter, float keep_prob,
                     MapData& out);
int validate_map(const msim_map& map);
int build_quad_tree(const float* pos, uint32_t n, float width, float height, uint32_t max_depth, uint32_t node_cap,
                    void* nodes_out, uint32_t node_capacity, void* links_out, uint32_t* nodes_used);

// Counter-based draws shared by every deterministic initializer: splitmix64 output
// function (Steele, Lea, Flood 2014) applied twice, keyed by (seed, stream, i).
inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
inline uint64_t draw(uint64_t seed, uint64_t stream, uint64_t i) {
    return splitmix64(splitmix64(seed + 0x632BE59BD9B4E019ULL * stream) + i);
}

}  // namespace msim

struct msim_map_buf {
    msim::MapData data;
};
