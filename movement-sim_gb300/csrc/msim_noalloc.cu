// msim_query_neighbours_noalloc: the radius neighbour query (the index rebuild
// and query of msim_step with MSIM_STEP_NEIGHBOURS) for positions the caller
// already holds on the device, without allocating any memory.
//
// Who needs this: callers that cannot call cudaMalloc at the point where they
// want neighbour sets.  cudaMalloc may synchronise the whole device and is not
// permitted while the calling thread is capturing a stream into a CUDA graph; a
// host application that hands all device memory to its own pool at start-up, or
// a tick loop that must never block in the allocator, cannot create an msim
// context (which allocates its buffers in msim_create and its export staging on
// first use).  This entry point takes device pointers for its inputs and
// outputs and keeps every intermediate (keys, radix-sort ping-pong buffers,
// digit histograms, look-back flags, tile ranges, a status word) in one
// file-scope __device__ array of fixed size, so it calls no cudaMalloc,
// cudaFree or other allocating routine.
//
// The array is shared by every call on a device and keeps the last call's
// contents; each call clears what must start at zero.  Calls whose GPU work
// overlaps (two streams, or two host threads) race on the array: serialise them.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "msim_internal.h"
#include "msim_kernels.cuh"

namespace msim {
namespace {

// Capacity: MSIM_NOALLOC_MAX_ENTITIES entities, tiles up to 512 x 512 (9 bits per axis).
constexpr uint32_t kMaxN = MSIM_NOALLOC_MAX_ENTITIES;
constexpr uint32_t kMaxBits = 9;
constexpr uint32_t kMaxKeys = 1u << (2 * kMaxBits);
constexpr uint32_t kMaxSortTiles = (kMaxN + kSortTile - 1) / kSortTile;
// word offsets inside the scratch array
constexpr size_t kOffKey = 0;
constexpr size_t kOffSk0 = kOffKey + kMaxN;
constexpr size_t kOffSv0 = kOffSk0 + kMaxN;
constexpr size_t kOffSk1 = kOffSv0 + kMaxN;
constexpr size_t kOffSv1 = kOffSk1 + kMaxN;
constexpr size_t kOffHist = kOffSv1 + kMaxN;
constexpr size_t kOffTickets = kOffHist + kMaxPasses * kRadix;
constexpr size_t kOffStatus = kOffTickets + 64;
constexpr size_t kOffLookback = kOffStatus + 64;
constexpr size_t kOffRanges = kOffLookback + (size_t)kMaxPasses * kMaxSortTiles * kRadix;
constexpr size_t kScratchWords = kOffRanges + 2ull * kMaxKeys;  // ~7.5 MB

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// The query, one thread per sorted position, writing each entity's count and
// ascending id list straight into the caller's id-indexed outputs.
__global__ __launch_bounds__(kQueryThreads) void k_noalloc_query(const uint32_t* __restrict__ sorted_id,
                                                                 const float2* __restrict__ pos,
                                                                 const uint2* __restrict__ ranges, TileGrid g,
                                                                 uint32_t n, uint32_t cap,
                                                                 uint32_t* __restrict__ count_out,
                                                                 uint32_t* __restrict__ idx_out) {
    extern __shared__ uint32_t s_list[];
    const uint32_t tid = threadIdx.x;
    const uint32_t p = blockIdx.x * kQueryThreads + tid;
    if (p >= n) return;
    const uint32_t s = sorted_id[p];
    if (s >= n) return;
    const float2 me = pos[s];
    // margin for the rounding of me -/+ reach at this position's magnitude
    const float mag = fmaxf(fabsf(me.x), fabsf(me.y));
    const float reach = __fadd_rn(__fmul_rn(g.radius, 1.00000095367431640625f), __fmul_rn(mag, 1.9073486328125e-6f));
    const uint32_t x0 = tile_coord(__fsub_rn(me.x, reach), g.inv_cell, g.tiles_x);
    const uint32_t x1 = tile_coord(__fadd_rn(me.x, reach), g.inv_cell, g.tiles_x);
    const uint32_t y0 = tile_coord(__fsub_rn(me.y, reach), g.inv_cell, g.tiles_y);
    const uint32_t y1 = tile_coord(__fadd_rn(me.y, reach), g.inv_cell, g.tiles_y);
    uint32_t count = 0;
    for (uint32_t ty = y0; ty <= y1; ty++) {
        for (uint32_t tx = x0; tx <= x1; tx++) {
            const uint2 rg = ranges[morton2(tx, ty)];
            const uint32_t qend = rg.y < n ? rg.y : n;
            for (uint32_t q = rg.x; q < qend; q++) {
                const uint32_t o = sorted_id[q];
                if (o == s || o >= n) continue;
                if (!in_range(pos[o], me, g.radius)) continue;
                if (cap) {
                    const uint32_t m = count < cap ? count : cap;
                    if (m < cap || o < s_list[(cap - 1) * kQueryThreads + tid]) {
                        uint32_t j = m < cap ? m : cap - 1;
                        while (j > 0) {
                            const uint32_t prev = s_list[(j - 1) * kQueryThreads + tid];
                            if (prev <= o) break;
                            s_list[j * kQueryThreads + tid] = prev;
                            j--;
                        }
                        s_list[j * kQueryThreads + tid] = o;
                    }
                }
                count++;
            }
        }
    }
    count_out[s] = count;
    if (cap) {
        const uint32_t kept = count < cap ? count : cap;
        uint32_t* dst = idx_out + (size_t)s * cap;
        for (uint32_t j = 0; j < cap; j++) dst[j] = j < kept ? s_list[j * kQueryThreads + tid] : MSIM_NO_NEIGHBOUR;
    }
}

// Per-device set-up: the scratch array's device address (the host-side symbol is
// only a stand-in, never a usable device pointer) and the query's shared-memory limit.
struct DeviceSlot {
    bool ready = false;
    uint32_t* scratch = nullptr;
    int sms = 0;
};
std::mutex g_setup_mutex;
DeviceSlot g_slots[64];

int setup_device(int dev, DeviceSlot** out) {
    if (dev < 0 || dev >= 64) return fail(MSIM_ERR_INVALID, "device ordinal out of range for the no-allocation path");
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    DeviceSlot& slot = g_slots[dev];
    if (!slot.ready) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(MSIM_ERR_CUDA, std::string("cudaGetSymbolAddress(no-allocation scratch) failed: ") +
                                           cudaGetErrorString(e));
        e = cudaFuncSetAttribute(k_noalloc_query, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(kMaxCap * kQueryThreads * sizeof(uint32_t)));
        if (e != cudaSuccess)
            return fail(MSIM_ERR_CUDA, std::string("cudaFuncSetAttribute failed: ") + cudaGetErrorString(e));
        e = cudaDeviceGetAttribute(&slot.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(MSIM_ERR_CUDA, std::string("cudaDeviceGetAttribute failed: ") + cudaGetErrorString(e));
        slot.scratch = static_cast<uint32_t*>(ptr);
        slot.ready = true;
    }
    *out = &slot;
    return MSIM_OK;
}

}  // namespace
}  // namespace msim

using namespace msim;

extern "C" int msim_query_neighbours_noalloc(const float* d_pos, uint32_t n, float world_w, float world_h,
                                             float radius, uint32_t cap, uint32_t* d_count, uint32_t* d_idx,
                                             uint32_t* d_status, void* stream) {
    if (n > kMaxN)
        return fail(MSIM_ERR_INVALID, "n = " + std::to_string(n) + " exceeds the no-allocation limit of " +
                                          std::to_string(kMaxN) + " entities");
    if (cap > kMaxCap) return fail(MSIM_ERR_INVALID, "cap must be <= " + std::to_string(kMaxCap));
    if (!std::isfinite(radius) || radius < 0.f) return fail(MSIM_ERR_INVALID, "radius must be finite and >= 0");
    if (!(world_w > 0.f) || !(world_h > 0.f) || !std::isfinite(world_w) || !std::isfinite(world_h))
        return fail(MSIM_ERR_INVALID, "world_w and world_h must be positive and finite");
    if (n && (!d_pos || !d_count || (cap && !d_idx)))
        return fail(MSIM_ERR_INVALID, "d_pos, d_count (and d_idx when cap > 0) are required");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MSIM_ERR_CUDA, std::string("cudaGetDevice failed: ") + cudaGetErrorString(e));
    DeviceSlot* slot = nullptr;
    int rc = setup_device(dev, &slot);
    if (rc != MSIM_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* w = slot->scratch;
    uint32_t* status = w + kOffStatus;
    if (cudaMemsetAsync(status, 0, sizeof(uint32_t), s) != cudaSuccess) return fail(MSIM_ERR_CUDA, "cudaMemsetAsync failed");
    if (n == 0) {
        if (d_status && cudaMemcpyAsync(d_status, status, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return fail(MSIM_ERR_CUDA, "cudaMemcpyAsync failed");
        return MSIM_OK;
    }

    // tile grid: at most 512 x 512 tiles so the ranges fit the scratch array
    const double cell_min = std::max((double)world_w, (double)world_h) / (double)(1u << kMaxBits) * (1.0 + 1e-6);
    double cell = std::max(2.0 * (double)radius * (1.0 + 0x1p-20),
                           4.0 * std::sqrt((double)world_w * (double)world_h / (double)n));
    cell = std::max(std::max(cell, cell_min), 1e-3);
    TileGrid g{};
    g.tiles_x = (uint32_t)std::max(1.0, std::ceil((double)world_w / cell));
    g.tiles_y = (uint32_t)std::max(1.0, std::ceil((double)world_h / cell));
    uint32_t bits = 1;
    while ((1u << bits) < std::max(g.tiles_x, g.tiles_y)) bits++;
    g.bits = bits;
    g.inv_cell = (float)(1.0 / cell);
    g.radius = radius;
    g.d2_limit = sqrt_limit(radius);
    g.reach = radius;  // the query below widens it per position
    g.ybits = 0;       // keys are tile codes only
    g.ybands = 1.f;
    const uint32_t passes = (2 * bits + 7) / 8;
    const uint32_t sort_tiles = (n + kSortTile - 1) / kSortTile;
    const size_t keys = (size_t)1 << (2 * bits);

    StepLaunch a{};
    a.st.pos = const_cast<float2*>(reinterpret_cast<const float2*>(d_pos));  // read only: ticks = 0
    a.n = n;
    a.ticks = 0;
    a.key = w + kOffKey;
    a.hist = w + kOffHist;
    a.grid = g;
    a.passes = passes;
    a.err = status;
    long long blocks = (long long)std::max(1, slot->sms) * 8;
    long long need = (n + kStepThreads - 1) / kStepThreads;
    a.blocks = (int)std::max(1LL, std::min(blocks, need));

    bool ok = cudaMemsetAsync(w + kOffHist, 0, sizeof(uint32_t) * kMaxPasses * kRadix, s) == cudaSuccess;
    ok = ok && launch_step(s, a) == cudaSuccess;
    ok = ok && cudaMemsetAsync(w + kOffLookback, 0, sizeof(uint32_t) * (size_t)passes * sort_tiles * kRadix, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(w + kOffTickets, 0, sizeof(uint32_t) * kMaxPasses, s) == cudaSuccess;
    uint32_t* sk[2] = {w + kOffSk0, w + kOffSk1};
    uint32_t* sv[2] = {w + kOffSv0, w + kOffSv1};
    for (uint32_t ps = 0; ok && ps < passes; ps++) {
        const uint32_t* kin = ps == 0 ? w + kOffKey : sk[(ps - 1) & 1];
        const uint32_t* vin = ps == 0 ? nullptr : sv[(ps - 1) & 1];
        ok = launch_onesweep(s, kin, vin, sk[ps & 1], sv[ps & 1], n, 8u * ps, w + kOffHist + ps * kRadix,
                             w + kOffLookback + (size_t)ps * sort_tiles * kRadix, w + kOffTickets + ps,
                             status) == cudaSuccess;
    }
    const uint32_t* sorted_key = sk[(passes - 1) & 1];
    const uint32_t* sorted_id = sv[(passes - 1) & 1];
    uint2* ranges = reinterpret_cast<uint2*>(w + kOffRanges);
    ok = ok && cudaMemsetAsync(ranges, 0, sizeof(uint2) * keys, s) == cudaSuccess;
    ok = ok && launch_ranges(s, sorted_key, n, ranges, (uint32_t)keys) == cudaSuccess;
    if (ok) {
        k_noalloc_query<<<(n + kQueryThreads - 1) / kQueryThreads, kQueryThreads,
                          (size_t)cap * kQueryThreads * sizeof(uint32_t), s>>>(
            sorted_id, reinterpret_cast<const float2*>(d_pos), ranges, g, n, cap, d_count, d_idx);
        ok = cudaGetLastError() == cudaSuccess;
    }
    if (ok && d_status)
        ok = cudaMemcpyAsync(d_status, status, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s) == cudaSuccess;
    if (!ok) return fail(MSIM_ERR_CUDA, std::string("no-allocation neighbour query: ") + cudaGetErrorString(cudaGetLastError()));
    return MSIM_OK;
}
